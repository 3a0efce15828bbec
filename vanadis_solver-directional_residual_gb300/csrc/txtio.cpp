// txtio.cpp -- the reference's text outputs of a time step, host side.
//
//   T_sssss.TXT           x, y, z and T * scale of every node, one node per
//                         line in Fortran format (e12.5, 2x, e12.5, 2x,
//                         e12.5, 2x, e12.5)  (vanadis_full_DR_OpenMP_timing
//                         .for:797-806, scale 1d6: kg/m^3 -> mg/m^3)
//   X_sssss_iii.TXT       the 2-D slices vanadis_files (:1089-1184) splits
//   Y_sssss_iii.TXT       from it: per x plane (y, z, s), per y row (z, x, s),
//   Z_sssss_iii.TXT       per z plane (y, x, s), format (e12.5, 2x, e12.5,
//                         2x, e12.5)
//
// Every line has a fixed width (54 or 40 characters and '\n'), so the text
// of a whole file is formatted by several host threads straight into one
// buffer at known offsets and written with one fwrite.  Fortran's Ew.d edit
// of a value is "0." followed by its d significant digits and the decimal
// exponent that goes with them: the digits come from the C library's
// correctly rounded conversion (round to nearest, ties to even on exact
// binary ties), the layout follows the Fortran standard's Ew.d rule
// (E+ee for |exponent| <= 99, +eee beyond).  The slices are formatted from
// the same doubles as the T file: rounding a value to 5 digits, reading it
// back and rounding again gives the same digits, so this equals splitting
// the written T file as the reference does.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "vdr.h"

namespace vdr {
void set_error(const std::string &msg);

namespace {

constexpr int W = 12;           // e12.5
constexpr int LINE4 = 4 * W + 3 * 2 + 1;
constexpr int LINE3 = 3 * W + 2 * 2 + 1;

// Fortran E12.5 of v into o[0..11] (no terminator).
void fmt_e12_5(double v, char *o) {
  if (std::isnan(v)) {
    std::memcpy(o, "         NaN", W);
    return;
  }
  if (std::isinf(v)) {
    std::memcpy(o, v < 0 ? "   -Infinity" : "    Infinity", W);
    return;
  }
  char b[40];
  std::snprintf(b, sizeof b, "%.4e", v);  // [-]d.dddde(+|-)xx[x]
  const char *p = b;
  const bool neg = *p == '-';
  if (neg) p++;
  const char *e = std::strchr(p, 'e');
  const int ex = e ? std::atoi(e + 1) : 0;
  const int fe = v == 0.0 ? 0 : ex + 1;  // 0.ddddd x 10^fe
  o[0] = neg ? '-' : ' ';
  o[1] = '0';
  o[2] = '.';
  o[3] = p[0];
  std::memcpy(o + 4, p + 2, 4);
  const int a = fe < 0 ? -fe : fe;
  if (a <= 99) {
    o[8] = 'E';
    o[9] = fe < 0 ? '-' : '+';
    o[10] = static_cast<char>('0' + a / 10);
    o[11] = static_cast<char>('0' + a % 10);
  } else {
    o[8] = fe < 0 ? '-' : '+';
    o[9] = static_cast<char>('0' + a / 100);
    o[10] = static_cast<char>('0' + (a / 10) % 10);
    o[11] = static_cast<char>('0' + a % 10);
  }
}

// Fixed-width lines [0, n) formatted by up to hardware_concurrency threads.
template <typename F>
void parallel_lines(long n, F &&line) {
  unsigned nt = std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  if (n < 65536) nt = 1;
  if ((long)nt > n) nt = n > 0 ? (unsigned)n : 1u;
  std::vector<std::thread> pool;
  const long chunk = (n + nt - 1) / nt;
  long inline_from = n;  // chunks no thread could be started for
  for (unsigned k = 1; k < nt; k++) {
    const long i0 = k * chunk, i1 = std::min(n, i0 + chunk);
    if (i0 >= i1) break;
    try {
      pool.emplace_back([=, &line] {
        for (long i = i0; i < i1; i++) line(i);
      });
    } catch (...) {
      inline_from = i0;
      break;
    }
  }
  for (long i = 0; i < std::min(n, chunk); i++) line(i);
  for (long i = inline_from; i < n; i++) line(i);
  for (auto &t : pool) t.join();
}

void put3(char *l, double a, double b, double c) {
  fmt_e12_5(a, l);
  l[12] = l[13] = ' ';
  fmt_e12_5(b, l + 14);
  l[26] = l[27] = ' ';
  fmt_e12_5(c, l + 28);
}

int write_file(const std::string &path, const std::vector<char> &buf) {
  FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) {
    set_error("cannot open " + path + " for writing");
    return VDR_IO_ERROR;
  }
  const size_t w = buf.empty() ? 0 : std::fwrite(buf.data(), 1, buf.size(), f);
  const int c = std::fclose(f);
  if (w != buf.size() || c != 0) {
    set_error("write to " + path + " failed");
    return VDR_IO_ERROR;
  }
  return VDR_OK;
}

std::string join(const char *dir, const char *name) {
  std::string s = dir ? dir : "";
  if (!s.empty() && s.back() != '/') s += '/';
  return s + name;
}

}  // namespace
}  // namespace vdr

using namespace vdr;

extern "C" {

int vdr_format_result_txt(char *buf, long nnode, const double *xx,
                          const double *yy, const double *zz, const double *t,
                          double scale) {
  if (!buf || nnode < 0 || (nnode > 0 && (!xx || !yy || !zz || !t))) {
    set_error("vdr_format_result_txt: bad arguments");
    return VDR_BAD_ARGUMENT;
  }
  parallel_lines(nnode, [&](long i) {
    char *l = buf + (size_t)i * LINE4;
    put3(l, xx[i], yy[i], zz[i]);
    l[40] = l[41] = ' ';
    fmt_e12_5(t[i] * scale, l + 42);
    l[54] = '\n';
  });
  return VDR_OK;
}

int vdr_write_result_txt(const char *dir, int step, long nnode,
                         const double *xx, const double *yy, const double *zz,
                         const double *t, double scale) {
  if (step < 0 || step > 99999 || nnode < 0 ||
      (nnode > 0 && (!xx || !yy || !zz || !t))) {
    set_error("vdr_write_result_txt: bad arguments (step 0..99999)");
    return VDR_BAD_ARGUMENT;
  }
  std::vector<char> buf;
  try {
    buf.resize((size_t)nnode * LINE4);
  } catch (...) {
    set_error("vdr_write_result_txt: out of host memory");
    return VDR_IO_ERROR;
  }
  int st = vdr_format_result_txt(buf.data(), nnode, xx, yy, zz, t, scale);
  if (st) return st;
  char name[32];
  std::snprintf(name, sizeof name, "T_%05d.TXT", step);
  return write_file(join(dir, name), buf);
}

int vdr_write_slices_txt(const char *dir, int step, int nax, int nay, int naz,
                         const double *xx, const double *yy, const double *zz,
                         const double *t, double scale) {
  if (step < 0 || step > 99999 || nax < 1 || nay < 1 || naz < 1 ||
      nax > 999 || nay > 999 || naz > 999 || !xx || !yy || !zz || !t) {
    set_error("vdr_write_slices_txt: bad arguments (step 0..99999, 1..999 "
              "nodes per axis: the file names carry i3.3 plane numbers)");
    return VDR_BAD_ARGUMENT;
  }
  const long x = nax, y = nay, z = naz;
  std::vector<char> buf;
  try {
    buf.reserve((size_t)std::max(x * y, std::max(x * z, y * z)) * LINE3);
  } catch (...) {
    set_error("vdr_write_slices_txt: out of host memory");
    return VDR_IO_ERROR;
  }
  char name[32];
  // X_: plane j = 1..x, nodes x (i - 1) + j for i = 1..y z: (y, z, s)
  for (long j = 1; j <= x; j++) {
    buf.resize((size_t)(y * z) * LINE3);
    parallel_lines(y * z, [&](long i) {
      const long n = x * i + j - 1;
      char *l = buf.data() + (size_t)i * LINE3;
      put3(l, yy[n], zz[n], t[n] * scale);
      l[40] = '\n';
    });
    std::snprintf(name, sizeof name, "X_%05d_%03ld.TXT", step, j);
    if (int st = write_file(join(dir, name), buf)) return st;
  }
  // Y_: row j = 1..y, nodes i + x (j - 1) + x y (k - 1) in plane order: (z, x, s)
  for (long j = 1; j <= y; j++) {
    buf.resize((size_t)(x * z) * LINE3);
    parallel_lines(x * z, [&](long i) {
      const long k = i / x, ii = i % x;
      const long n = ii + x * (j - 1) + x * y * k;
      char *l = buf.data() + (size_t)i * LINE3;
      put3(l, zz[n], xx[n], t[n] * scale);
      l[40] = '\n';
    });
    std::snprintf(name, sizeof name, "Y_%05d_%03ld.TXT", step, j);
    if (int st = write_file(join(dir, name), buf)) return st;
  }
  // Z_: plane j = 1..z, nodes i + x y (j - 1): (y, x, s)
  for (long j = 1; j <= z; j++) {
    buf.resize((size_t)(x * y) * LINE3);
    parallel_lines(x * y, [&](long i) {
      const long n = i + x * y * (j - 1);
      char *l = buf.data() + (size_t)i * LINE3;
      put3(l, yy[n], xx[n], t[n] * scale);
      l[40] = '\n';
    });
    std::snprintf(name, sizeof name, "Z_%05d_%03ld.TXT", step, j);
    if (int st = write_file(join(dir, name), buf)) return st;
  }
  return VDR_OK;
}

}  // extern "C"
