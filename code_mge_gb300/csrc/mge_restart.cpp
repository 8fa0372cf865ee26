// mge_restart.cpp -- the reference's restart file as text: write_solut
// (wsolut.f90:49-92) and read_solut (rsolut.f90:1-41).
//
// Per block, in the order of the block list:
//   "(5I5)"    code, low(1:4), upp(1:4)   -- 9 integers, 5 per line
//   "(5f16.7)" w(low1:upp1, low2:upp2, low3:upp3, low4:upp4), i fastest,
//              5 values per line (format reversion starts a new line)
// with low = (0,0,0,1) and upp = (ib,jb,kb,5).  A field that does not fit its
// width is written as asterisks, as Fortran does.  Reading checks the code
// and upp(1:4) against the block, as read_solut does before it stops on a
// mismatch, and reads every value from its own 16 columns.
//
// Only host code: these functions run without a GPU.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/mge_gpu.h"

namespace {

// Fortran I5
void put_i5(std::string& o, int v) {
  char t[32];
  const int n = std::snprintf(t, sizeof t, "%5d", v);
  o += (n > 5) ? "*****" : t;
}

// Fortran F16.7: the value rounded to 7 decimals, right-justified in 16
// columns; asterisks when it needs more; NaN and Infinity spelled as
// gfortran writes them
void put_f16_7(std::string& o, double v) {
  char t[64];
  if (std::isnan(v)) {
    std::snprintf(t, sizeof t, "%16s", "NaN");
  } else if (std::isinf(v)) {
    std::snprintf(t, sizeof t, "%16s", v > 0 ? "Infinity" : "-Infinity");
  } else {
    const int n = std::snprintf(t, sizeof t, "%16.7f", v);
    if (n > 16) {
      o += "****************";
      return;
    }
  }
  o += t;
}

// one text line starting at *pos (without its end of line); advances *pos
bool next_line(const char* s, long long len, long long* pos, const char** b, long long* n) {
  if (*pos >= len) return false;
  long long e = *pos;
  while (e < len && s[e] != '\n') e++;
  *b = s + *pos;
  *n = e - *pos;
  if (*n > 0 && (*b)[*n - 1] == '\r') (*n)--;
  *pos = (e < len) ? e + 1 : e;
  return true;
}

// a fixed-width field as an integer or a double; false when it is not one
bool field_int(const char* f, int width, int* out) {
  char t[64];
  std::memcpy(t, f, width);
  t[width] = 0;
  char* end = nullptr;
  const long v = std::strtol(t, &end, 10);
  while (end && *end == ' ') end++;
  if (!end || *end || end == t) return false;
  *out = (int)v;
  return true;
}

bool field_double(const char* f, int width, double* out) {
  char t[64];
  std::memcpy(t, f, width);
  t[width] = 0;
  const char* p = t;
  while (*p == ' ') p++;
  if (!*p || *p == '*') return false;
  char* end = nullptr;
  const double v = std::strtod(p, &end);
  while (end && *end == ' ') end++;
  if (!end || *end) return false;
  *out = v;
  return true;
}

}  // namespace

extern "C" long long mge_restart_format(int code, int ib, int jb, int kb, const double* w, char* buf, long long cap) {
  if (ib < 0 || jb < 0 || kb < 0 || (buf && !w)) return MGE_EBADCFG;
  const long long nval = 5LL * (ib + 1) * (jb + 1) * (kb + 1);
  std::string o;
  o.reserve((size_t)(nval * 16 + nval / 5 + 64));
  const int head[9] = {code, 0, 0, 0, 1, ib, jb, kb, 5};
  for (int q = 0; q < 9; q++) {
    put_i5(o, head[q]);
    if (q == 4 || q == 8) o += '\n';
  }
  for (long long q = 0; q < nval; q++) {
    put_f16_7(o, w ? w[q] : 0.0);
    if (q % 5 == 4 || q == nval - 1) o += '\n';
  }
  const long long need = (long long)o.size();
  if (buf && cap > 0) {
    const long long n = need < cap - 1 ? need : cap - 1;
    std::memcpy(buf, o.data(), (size_t)n);
    buf[n] = 0;
  }
  return need;
}

extern "C" long long mge_restart_parse(const char* text, long long len, int code, int ib, int jb, int kb, double* w) {
  if (!text || !w || len < 0) return MGE_EBADCFG;
  long long pos = 0;
  const char* ln;
  long long n;
  int head[9], got = 0;
  while (got < 9) {
    if (!next_line(text, len, &pos, &ln, &n)) return MGE_EBADCFG;
    for (long long f = 0; f + 5 <= n && got < 9 && f < 25; f += 5)
      if (!field_int(ln + f, 5, &head[got++])) return MGE_EBADCFG;
  }
  // rsolut.f90:27-32: the code and the upper bounds must be this block's
  if (head[0] != code || head[5] != ib || head[6] != jb || head[7] != kb || head[8] != 5) return MGE_EBADCFG;
  if (head[1] != 0 || head[2] != 0 || head[3] != 0 || head[4] != 1) return MGE_EBADCFG;
  const long long nval = 5LL * (ib + 1) * (jb + 1) * (kb + 1);
  long long q = 0;
  while (q < nval) {
    if (!next_line(text, len, &pos, &ln, &n)) return MGE_EBADCFG;
    for (long long f = 0; f + 16 <= n && q < nval && f < 80; f += 16)
      if (!field_double(ln + f, 16, &w[q++])) return MGE_EBADCFG;
  }
  return pos;
}
