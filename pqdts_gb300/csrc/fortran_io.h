// Host-side formats of pqdts_omp.x that the drop-in must keep:
//   * gfortran list-directed output (PRINT *): the stdout lines that pqdts.py
//     parses (`iter` line token 4 = objective, pqdts.py:77-78), the timing
//     and status files (pqdts.f90:159-186, 2208-2223);
//   * gfortran sequential unformatted records (4-byte length markers, records
//     above 2147483639 bytes split into sub-records with signed markers) for
//     the stage, final and restart files (pqdts.f90:1848-1875, 2150-2160,
//     2187-2197).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace pqdts {

// One list-directed record.  Items are appended in order; numeric items are
// right-justified in gfortran's widths (integer(4): 11, integer(8): 20,
// real(8): 25) after a one-blank separator, character items are written
// as-is with a blank only when they follow a numeric item.
class ListLine {
 public:
  ListLine& s(const std::string& t) {
    if (!first_ && !prev_char_) buf_ += ' ';
    buf_ += t;
    prev_char_ = true;
    first_ = false;
    return *this;
  }
  ListLine& i4(long long v) { return num(fmt("%11lld", v)); }
  ListLine& i8(long long v) { return num(fmt("%20lld", v)); }
  ListLine& r8(double v) { return num(real8(v)); }
  const std::string& str() const { return buf_; }
  void print(FILE* f = stdout) const { fprintf(f, "%s\n", buf_.c_str()); }

  // gfortran's G-style list-directed REAL(8): 17 significant digits, fixed
  // form for 0.1 <= |v| < 1e17 followed by 5 blanks, else E form with a
  // three-digit exponent; 25 characters.
  static std::string real8(double v) {
    char b[80];
    if (std::isnan(v)) return fmt("%25s", "NaN");
    if (std::isinf(v)) return fmt("%25s", v > 0 ? "Infinity" : "-Infinity");
    if (v == 0.0) {
      snprintf(b, sizeof b, "%20.16f     ", v);
      return b;
    }
    char e[80];
    snprintf(e, sizeof e, "%.16e", v);
    const char* ep = strchr(e, 'e');
    int ex = atoi(ep + 1);
    int k = ex + 1;
    if (k >= 0 && k <= 17) {
      snprintf(b, sizeof b, "%20.*f     ", 17 - k, v);
      return b;
    }
    std::string mant(e, (size_t)(ep - e));
    char t[80];
    snprintf(t, sizeof t, "%sE%c%03d", mant.c_str(), ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
    return fmt("%25s", t);
  }

 private:
  template <typename... A>
  static std::string fmt(const char* f, A... a) {
    char b[128];
    snprintf(b, sizeof b, f, a...);
    return b;
  }
  ListLine& num(const std::string& t) {
    if (!first_) buf_ += ' ';
    buf_ += t;
    first_ = false;
    prev_char_ = false;
    return *this;
  }
  std::string buf_ = " ";
  bool first_ = true;
  bool prev_char_ = true;
};

inline void write_record(FILE* f, const void* data, size_t bytes) {
  const size_t kMax = 2147483639u;
  const char* p = static_cast<const char*>(data);
  size_t left = bytes;
  bool first = true;
  do {
    size_t chunk = left < kMax ? left : kMax;
    bool more = left > chunk;
    int32_t lead = (int32_t)chunk, tail = (int32_t)chunk;
    if (more) lead = -lead;
    if (!first) tail = -tail;
    fwrite(&lead, 4, 1, f);
    if (chunk) fwrite(p, 1, chunk, f);
    fwrite(&tail, 4, 1, f);
    p += chunk;
    left -= chunk;
    first = false;
  } while (left > 0);
}

inline bool read_record(FILE* f, std::vector<char>& out) {
  out.clear();
  for (;;) {
    int32_t lead, tail;
    if (fread(&lead, 4, 1, f) != 1) return false;
    size_t len = (size_t)(lead < 0 ? -(int64_t)lead : (int64_t)lead);
    size_t at = out.size();
    out.resize(at + len);
    if (len && fread(out.data() + at, 1, len, f) != len) return false;
    if (fread(&tail, 4, 1, f) != 1) return false;
    if (lead >= 0) return true;
  }
}

// Stage / final file (pqdts.f90:2146-2160, 2183-2197): M, N, D, localrows
// (int64), rank (int32), X (M,N) column-major float64.
inline bool write_state_file(const char* path, int64_t M, int64_t N, int64_t D, int32_t rank, const double* X) {
  FILE* f = fopen(path, "wb");
  if (!f) return false;
  write_record(f, &M, 8);
  write_record(f, &N, 8);
  write_record(f, &D, 8);
  write_record(f, &M, 8);
  write_record(f, &rank, 4);
  write_record(f, X, (size_t)M * (size_t)N * 8);
  return fclose(f) == 0;
}

inline std::string stage_file_name(int rank, int oiter) {
  char b[64];
  snprintf(b, sizeof b, "rank_%6d_oiter%6d.dat", rank, oiter);
  return b;
}

inline std::string final_file_name(int rank) {
  char b[64];
  snprintf(b, sizeof b, "rank_%6d_final.dat", rank);
  return b;
}

// `write (str, *) "timing_", rank, ".out"` after adjustl/trim.
inline std::string listed_file_name(const char* stem, int rank) {
  ListLine l;
  l.s(stem).i4(rank).s(".out");
  std::string s = l.str();
  size_t p = s.find_first_not_of(' ');
  return p == std::string::npos ? s : s.substr(p);
}

}  // namespace pqdts
