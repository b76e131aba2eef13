// fileio.cpp -- the reference's result files, byte-compatible, on the host.
//
//  * wf<i>.bin: one Fortran unformatted sequential record holding
//    psi(1:dim) as complex(8) (write_wf / read_wf, input_param.f90:119-184).
//    Record markers are 4-byte little-endian byte counts before and after
//    the data (gfortran's default).  A record longer than 2147483639 bytes is
//    split into subrecords of at most that length; the leading marker of
//    every subrecord but the last is negated (more follow) and the trailing
//    marker of every subrecord but the first is negated (some precede).
//  * energy.dat: one line per state, format (2ES24.15): dble(i), ene(i).
//  * alpha_beta_values_*.d: one line per DSF level, format (3I6, 8e23.15):
//    ex_i, n, itr, alpha(n), beta(n), norm1, E0, sztot
//    (get_expectation_values.f90:522-525, 570-573, 595-603).  The reference
//    writes level 1 of the -tmp.d file with (3I6, 7e23.15, I15), an I edit
//    descriptor for the real(8) sztot, which gfortran rejects at run time;
//    here every line, level 1 included, uses (3I6, 8e23.15), which the
//    list-directed read of DSFLan (source_DSFLan/main.f90:43-48) accepts.
//
// Fortran E and ES output is produced from the correctly rounded decimal
// expansion of printf: Ew.d prints 0.d1...dd with exponent e+1 where
// printf("%.{d-1}e") gives d1.d2...dd e; ESw.d is printf("%.{d}e").  The
// exponent field is E+dd for |exp| <= 99 and +ddd (no letter) for
// 99 < |exp| <= 999, as the Fortran standard prescribes when Ee is absent.
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/qs3g.h"

namespace qs3g {
void set_global_error(const std::string& msg);  // defined with the C ABI (capi.cu)
}

namespace {

int fail(int code, const std::string& msg) {
  qs3g::set_global_error(msg);
  return code;
}

constexpr int64_t kMaxSubrecord = 2147483639;  // gfortran's default subrecord limit

bool put_marker(FILE* f, int32_t v) {
  unsigned char b[4];
  const uint32_t u = (uint32_t)v;
  for (int k = 0; k < 4; ++k) b[k] = (unsigned char)((u >> (8 * k)) & 0xffu);
  return std::fwrite(b, 1, 4, f) == 4;
}

bool get_marker(FILE* f, int32_t& v) {
  unsigned char b[4];
  if (std::fread(b, 1, 4, f) != 4) return false;
  uint32_t u = 0;
  for (int k = 0; k < 4; ++k) u |= (uint32_t)b[k] << (8 * k);
  v = (int32_t)u;
  return true;
}

// Mantissa digits and decimal exponent of x rounded to `digits` significant
// digits: x = d1.d2...d_digits * 10^e.  Returns false for non-finite x.
bool decimal(double x, int digits, std::string& mant, int& e, bool& neg) {
  if (!std::isfinite(x)) return false;
  char buf[64];
  std::snprintf(buf, sizeof buf, "%.*e", digits - 1, x);
  const char* p = buf;
  neg = (*p == '-');
  if (neg) ++p;
  mant.clear();
  for (; *p && *p != 'e'; ++p)
    if (*p != '.') mant.push_back(*p);
  e = (*p == 'e') ? std::atoi(p + 1) : 0;
  return true;
}

std::string exponent_field(int e) {
  char buf[16];
  const int a = e < 0 ? -e : e;
  if (a <= 99) std::snprintf(buf, sizeof buf, "E%c%02d", e < 0 ? '-' : '+', a);
  else if (a <= 999) std::snprintf(buf, sizeof buf, "%c%03d", e < 0 ? '-' : '+', a);
  else return std::string();  // does not fit: the field becomes asterisks
  return buf;
}

std::string pad(const std::string& s, int w) {
  if ((int)s.size() > w) return std::string(w, '*');
  return std::string(w - s.size(), ' ') + s;
}

std::string nonfinite(double x, int w) {
  if (std::isnan(x)) return pad("NaN", w);
  const bool neg = x < 0;
  std::string s = (w >= 9) ? "Infinity" : "Inf";
  if (neg) s = "-" + s;
  else if (w > (int)s.size()) s = "+" + s;
  return pad(s, w);
}

}  // namespace

// Fortran Ew.d of x (w <= 64).
static std::string fortran_e(double x, int w, int d) {
  std::string m;
  int e;
  bool neg;
  if (!decimal(x, d, m, e, neg)) return nonfinite(x, w);
  const bool zero = (x == 0.0);
  const int ex = zero ? 0 : e + 1;
  const std::string ef = exponent_field(ex);
  if (ef.empty()) return std::string(w, '*');
  std::string body = "." + m + ef;
  // the optional leading zero is printed when the width allows it
  std::string s = std::string(neg ? "-" : "") + "0" + body;
  if ((int)s.size() > w) s = std::string(neg ? "-" : "") + body;
  return pad(s, w);
}

// Fortran ESw.d of x.
static std::string fortran_es(double x, int w, int d) {
  std::string m;
  int e;
  bool neg;
  if (!decimal(x, d + 1, m, e, neg)) return nonfinite(x, w);
  const int ex = (x == 0.0) ? 0 : e;
  const std::string ef = exponent_field(ex);
  if (ef.empty()) return std::string(w, '*');
  std::string s = std::string(neg ? "-" : "") + m.substr(0, 1) + "." + m.substr(1) + ef;
  return pad(s, w);
}

static std::string fortran_i(long long v, int w) { return pad(std::to_string(v), w); }

// Parse one real as list-directed input accepts it, including the exponent
// forms without a letter ("0.1+301") that E output produces.
static bool parse_real(const std::string& tok, double& v) {
  std::string t = tok;
  for (auto& c : t)
    if (c == 'd' || c == 'D' || c == 'q' || c == 'Q') c = 'e';
  // insert 'e' before a sign that follows a digit or '.' (exponent without letter)
  for (size_t k = 1; k < t.size(); ++k)
    if ((t[k] == '+' || t[k] == '-') && (std::isdigit((unsigned char)t[k - 1]) || t[k - 1] == '.')) {
      t.insert(k, "e");
      break;
    }
  char* end = nullptr;
  errno = 0;
  v = std::strtod(t.c_str(), &end);
  return end && *end == '\0' && end != t.c_str();
}

static std::vector<std::string> split_fields(const std::string& line) {
  std::vector<std::string> out;
  std::string cur;
  for (char c : line) {
    if (c == ' ' || c == '\t' || c == ',' || c == '\r' || c == '\n') {
      if (!cur.empty()) { out.push_back(cur); cur.clear(); }
    } else {
      cur.push_back(c);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

extern "C" {

int qs3g_write_wf(const char* path, const int64_t* dim, const qs3g_cplx* psi) {
  if (!path || !dim || *dim < 0 || (*dim > 0 && !psi)) return fail(QS3G_EINVAL, "qs3g_write_wf: bad argument");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(QS3G_EINVAL, std::string("qs3g_write_wf: cannot open ") + path);
  const int64_t total = *dim * (int64_t)sizeof(qs3g_cplx);
  const unsigned char* p = (const unsigned char*)psi;
  int64_t done = 0;
  bool ok = true;
  int part = 0;
  do {
    const int64_t len = std::min<int64_t>(kMaxSubrecord, total - done);
    const bool last = (done + len == total);
    ok = ok && put_marker(f, last ? (int32_t)len : -(int32_t)len);
    if (len > 0) ok = ok && std::fwrite(p + done, 1, (size_t)len, f) == (size_t)len;
    ok = ok && put_marker(f, part == 0 ? (int32_t)len : -(int32_t)len);
    done += len;
    ++part;
  } while (ok && done < total);
  ok = (std::fclose(f) == 0) && ok;
  return ok ? QS3G_OK : fail(QS3G_EINVAL, std::string("qs3g_write_wf: write failed for ") + path);
}

int qs3g_read_wf(const char* path, const int64_t* dim, qs3g_cplx* psi) {
  if (!path || !dim || *dim < 0 || (*dim > 0 && !psi)) return fail(QS3G_EINVAL, "qs3g_read_wf: bad argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(QS3G_EINVAL, std::string("qs3g_read_wf: cannot open ") + path);
  const int64_t want = *dim * (int64_t)sizeof(qs3g_cplx);
  unsigned char* p = (unsigned char*)psi;
  int64_t got = 0;
  bool more = true;
  while (more) {
    int32_t lead, trail;
    if (!get_marker(f, lead)) { std::fclose(f); return fail(QS3G_EINVAL, "qs3g_read_wf: truncated record marker"); }
    more = lead < 0;
    const int64_t len = lead < 0 ? -(int64_t)lead : lead;
    // read(10) psi(1:dim) takes the first dim values of the record
    const int64_t take = std::min<int64_t>(len, std::max<int64_t>(0, want - got));
    if (take > 0 && std::fread(p + got, 1, (size_t)take, f) != (size_t)take) {
      std::fclose(f);
      return fail(QS3G_EINVAL, "qs3g_read_wf: truncated record");
    }
    got += take;
    if (len > take && std::fseek(f, (long)(len - take), SEEK_CUR) != 0) {
      std::fclose(f);
      return fail(QS3G_EINVAL, "qs3g_read_wf: truncated record");
    }
    if (!get_marker(f, trail) || (trail < 0 ? -(int64_t)trail : trail) != len) {
      std::fclose(f);
      return fail(QS3G_EINVAL, "qs3g_read_wf: record markers disagree");
    }
  }
  std::fclose(f);
  if (got < want) return fail(QS3G_ERANGE, "qs3g_read_wf: record shorter than dim complex(8) values");
  return QS3G_OK;
}

int qs3g_write_energy(const char* path, const int* NOE, const double* ene) {
  if (!path || !NOE || *NOE < 0 || (*NOE > 0 && !ene)) return fail(QS3G_EINVAL, "qs3g_write_energy: bad argument");
  FILE* f = std::fopen(path, "w");
  if (!f) return fail(QS3G_EINVAL, std::string("qs3g_write_energy: cannot open ") + path);
  bool ok = true;
  for (int i = 1; i <= *NOE; ++i) {
    const std::string line = fortran_es((double)i, 24, 15) + fortran_es(ene[i - 1], 24, 15) + "\n";
    ok = ok && std::fputs(line.c_str(), f) >= 0;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? QS3G_OK : fail(QS3G_EINVAL, "qs3g_write_energy: write failed");
}

int qs3g_read_energy(const char* path, const int* NOE, double* ene) {
  if (!path || !NOE || *NOE < 0 || (*NOE > 0 && !ene)) return fail(QS3G_EINVAL, "qs3g_read_energy: bad argument");
  FILE* f = std::fopen(path, "r");
  if (!f) return fail(QS3G_EINVAL, std::string("qs3g_read_energy: cannot open ") + path);
  char buf[1024];
  int i = 0;
  while (i < *NOE && std::fgets(buf, sizeof buf, f)) {
    const auto fl = split_fields(buf);
    if (fl.empty()) continue;
    double dummy, e;
    if (fl.size() < 2 || !parse_real(fl[0], dummy) || !parse_real(fl[1], e)) {
      std::fclose(f);
      return fail(QS3G_EINVAL, "qs3g_read_energy: malformed line");
    }
    ene[i++] = e;
  }
  std::fclose(f);
  if (i < *NOE) return fail(QS3G_ERANGE, "qs3g_read_energy: fewer lines than NOE");
  return QS3G_OK;
}

int qs3g_write_alpha_beta(const char* path, const int* nlines, const int* ex_i, const int* itr,
                          const double* alpha, const double* beta2, const double* norm1, const double* E0,
                          const double* sztot, const int* append) {
  if (!path || !nlines || *nlines < 0 || !ex_i || !itr || !norm1 || !E0 || !sztot ||
      (*nlines > 0 && (!alpha || !beta2)))
    return fail(QS3G_EINVAL, "qs3g_write_alpha_beta: bad argument");
  FILE* f = std::fopen(path, (append && *append) ? "a" : "w");
  if (!f) return fail(QS3G_EINVAL, std::string("qs3g_write_alpha_beta: cannot open ") + path);
  bool ok = true;
  for (int n = 1; n <= *nlines; ++n) {
    std::string line = fortran_i(*ex_i, 6) + fortran_i(n, 6) + fortran_i(*itr, 6);
    line += fortran_e(alpha[n - 1], 23, 15) + fortran_e(beta2[n - 1], 23, 15) + fortran_e(*norm1, 23, 15) +
            fortran_e(*E0, 23, 15) + fortran_e(*sztot, 23, 15) + "\n";
    ok = ok && std::fputs(line.c_str(), f) >= 0;
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? QS3G_OK : fail(QS3G_EINVAL, "qs3g_write_alpha_beta: write failed");
}

int qs3g_read_alpha_beta(const char* path, const int* cap, double* alpha, double* beta2, double* norm1,
                         double* E0, double* sztot, int* nlines) {
  if (!path || !cap || *cap < 0 || !nlines) return fail(QS3G_EINVAL, "qs3g_read_alpha_beta: bad argument");
  FILE* f = std::fopen(path, "r");
  if (!f) return fail(QS3G_EINVAL, std::string("qs3g_read_alpha_beta: cannot open ") + path);
  char buf[4096];
  int n = 0;
  while (std::fgets(buf, sizeof buf, f)) {
    const auto fl = split_fields(buf);
    if (fl.empty()) continue;
    double v[8];
    if (fl.size() < 8) { std::fclose(f); return fail(QS3G_EINVAL, "qs3g_read_alpha_beta: short line"); }
    for (int k = 0; k < 8; ++k)
      if (!parse_real(fl[k], v[k])) { std::fclose(f); return fail(QS3G_EINVAL, "qs3g_read_alpha_beta: bad field"); }
    if (n < *cap) {
      if (alpha) alpha[n] = v[3];
      if (beta2) beta2[n] = v[4];
    }
    // the last line read wins, as in the reference's read loop
    if (norm1) *norm1 = v[5];
    if (E0) *E0 = v[6];
    if (sztot) *sztot = v[7];
    ++n;
  }
  std::fclose(f);
  *nlines = n;
  if (n > *cap) return fail(QS3G_ERANGE, "qs3g_read_alpha_beta: more lines than cap");
  return QS3G_OK;
}

// Fortran edit-descriptor output of one value, for callers writing their own
// files in the reference's formats: kind 0 = Ew.d, 1 = ESw.d.  out receives w
// characters and a terminating NUL (out must hold w + 1 bytes).
int qs3g_format_real(const double* x, const int* kind, const int* w, const int* d, char* out) {
  if (!x || !kind || !w || !d || !out || *w < 1 || *w > 64 || *d < 1 || *d > 30)
    return fail(QS3G_EINVAL, "qs3g_format_real: bad argument");
  const std::string s = (*kind == 1) ? fortran_es(*x, *w, *d) : fortran_e(*x, *w, *d);
  std::memcpy(out, s.data(), s.size());
  out[s.size()] = '\0';
  return QS3G_OK;
}

}  // extern "C"
