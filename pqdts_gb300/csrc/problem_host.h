// Host-side construction of a problem: F bands, P, the transposed CSR and
// the Hessian diagonal.  All of it is set-up work done once per problem, in
// O(nnz) (the reference's band build is O(D*nnz), pqdts.f90:1328-1364).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

namespace pqdts {

struct HostProblem {
  int64_t M = 0, N = 0, D = 0;
  double gam = 0.0;
  std::vector<int32_t> flo, fw;  // band start (-1 = empty row) and width
  std::vector<int64_t> foff;
  std::vector<double> fval;
  std::vector<double> P;         // (D, N) row-major
  std::vector<int64_t> tptr;     // transposed CSR over columns i of F
  std::vector<int32_t> tidx;
  std::vector<double> tval;
  std::vector<double> bdiag;     // full-space Hessian diagonal, one value per row i
  // F^T as dense bands over d (zero filled where column i is not in row d's
  // band): the mixed-precision tiled product's operand.
  std::vector<int32_t> tlo, tw;
  std::vector<int64_t> toff;
  std::vector<double> tbval;
  int64_t nnz() const { return (int64_t)fval.size(); }
};

// splitmix64 uniform [0,1) stream seeded with 23764 (the reference's seed,
// pqdts.f90:1116): stands in for gfortran's RANDOM_NUMBER.  The first N*D
// draws fill a random P (n fastest), the next M*N the initial random X whose
// row maxima give the first maxr (1565-1575).
struct SeededStream {
  uint64_t s = 23764;
  double next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
  }
};

inline void finish_offsets(HostProblem& h) {
  h.foff.assign(h.D, 0);
  int64_t tot = 0;
  for (int64_t d = 0; d < h.D; ++d) {
    h.foff[d] = tot;
    tot += h.fw[d];
  }
  h.fval.assign(tot, 0.0);
}

// Bands from COO: [min col, max col] per row, zero filled, duplicates
// overwrite in input order (pqdts.f90:1334-1363).
inline void bands_from_coo(HostProblem& h, int64_t nnz, const int32_t* row, const int32_t* col, const double* val) {
  h.flo.assign(h.D, -1);
  std::vector<int32_t> hi(h.D, -1);
  for (int64_t k = 0; k < nnz; ++k) {
    const int64_t d = row[k], i = col[k];
    if (d < 0 || d >= h.D || i < 0 || i >= h.M)
      throw std::invalid_argument("F entry " + std::to_string(k) + " out of range (row " + std::to_string(d) +
                                  ", col " + std::to_string(i) + ")");
    if (h.flo[d] < 0 || i < h.flo[d]) h.flo[d] = (int32_t)i;
    if (i > hi[d]) hi[d] = (int32_t)i;
  }
  h.fw.assign(h.D, 0);
  for (int64_t d = 0; d < h.D; ++d)
    if (h.flo[d] >= 0) h.fw[d] = hi[d] - h.flo[d] + 1;
  finish_offsets(h);
  for (int64_t k = 0; k < nnz; ++k) h.fval[h.foff[row[k]] + col[k] - h.flo[row[k]]] = val[k];
}

inline void bands_from_bands(HostProblem& h, const int64_t* lo, const int64_t* hi, const double* vals) {
  h.flo.assign(h.D, -1);
  h.fw.assign(h.D, 0);
  for (int64_t d = 0; d < h.D; ++d) {
    if (lo[d] < 0) continue;
    if (hi[d] < lo[d] || hi[d] >= h.M) throw std::invalid_argument("band " + std::to_string(d) + " out of range");
    h.flo[d] = (int32_t)lo[d];
    h.fw[d] = (int32_t)(hi[d] - lo[d] + 1);
  }
  finish_offsets(h);
  std::copy(vals, vals + h.fval.size(), h.fval.begin());
}

// fprob (pqdts.f90:188-206): Poisson pmf for mean < 50, Gaussian otherwise.
inline double fprob(double x, double mean) {
  const double pi = 4.0 * std::atan(1.0);
  if (mean < 50) {
    if (mean == 0 && x == 0) return 1.0;
    const double lf = std::lgamma(x + 1.0);
    return std::exp(std::fma(std::log(mean), x, -lf) - mean);
  }
  const double y = (x - mean) / std::sqrt(mean);
  return std::exp(-0.5 * (y * y)) / std::sqrt(mean) / std::sqrt(2 * pi);
}

// Internal F (pqdts.f90:1366-1466): row d (1-based i) has mean (D-i)^2 and
// keeps the window where fprob >= 1e-10; requires M == (D-1)^2.
inline void bands_internal(HostProblem& h) {
  if (h.M != (h.D - 1) * (h.D - 1)) throw std::invalid_argument("M is not (D-1)**2");
  h.flo.assign(h.D, -1);
  h.fw.assign(h.D, 0);
  std::vector<int64_t> mean_of(h.D);
  for (int64_t i = 1; i <= h.D; ++i) {
    const int64_t mean = (h.D - i) * (h.D - i);
    mean_of[i - 1] = mean;
    int64_t i0 = std::numeric_limits<int64_t>::max(), i1 = 0;
    for (int64_t j = std::max<int64_t>(1, mean); j <= h.M; ++j) {
      if (fprob((double)(j - 1), (double)mean) < 1e-10) break;
      i0 = std::min(j, i0);
      i1 = std::max(j, i1);
    }
    for (int64_t j = std::max<int64_t>(1, mean); j >= 1; --j) {
      if (fprob((double)(j - 1), (double)mean) < 1e-10) break;
      i0 = std::min(j, i0);
      i1 = std::max(j, i1);
    }
    if (i1 >= 1 && i0 <= h.M) {
      h.flo[i - 1] = (int32_t)(i0 - 1);
      h.fw[i - 1] = (int32_t)(i1 - i0 + 1);
    }
  }
  finish_offsets(h);
  for (int64_t d = 0; d < h.D; ++d)
    for (int64_t k = 0; k < h.fw[d]; ++k) h.fval[h.foff[d] + k] = fprob((double)(h.flo[d] + k), (double)mean_of[d]);
}

inline void P_from_coo(HostProblem& h, int64_t nnz, const int32_t* row, const int32_t* col, const double* val,
                       SeededStream& rng) {
  h.P.assign((size_t)h.D * h.N, 0.0);
  if (nnz < 0) {
    for (size_t k = 0; k < h.P.size(); ++k) h.P[k] = rng.next();
    return;
  }
  for (int64_t k = 0; k < nnz; ++k) {
    if (row[k] < 0 || row[k] >= h.D || col[k] < 0 || col[k] >= h.N)
      throw std::invalid_argument("P entry " + std::to_string(k) + " out of range");
    h.P[(size_t)row[k] * h.N + col[k]] = val[k];
  }
}

// Transposed CSR (ascending d per column i) and the full-space Hessian
// diagonal in the reference's order: 2*f^2 summed over ascending d, then
// +2*gamma on rows 1..M-1, then +2*gamma on rows 2..M (pqdts.f90:214-234).
inline void finish_problem(HostProblem& h) {
  if ((int64_t)h.M * h.N >= (int64_t)1 << 31) throw std::invalid_argument("M*N must be below 2^31");
  std::vector<int64_t> cnt(h.M + 1, 0);
  for (int64_t d = 0; d < h.D; ++d)
    if (h.fw[d] > 0) {
      cnt[h.flo[d]] += 1;
      cnt[h.flo[d] + h.fw[d]] -= 1;
    }
  h.tptr.assign(h.M + 1, 0);
  int64_t run = 0;
  for (int64_t i = 0; i < h.M; ++i) {
    run += cnt[i];
    h.tptr[i + 1] = h.tptr[i] + run;
  }
  h.tidx.assign(h.tptr[h.M], 0);
  h.tval.assign(h.tptr[h.M], 0.0);
  std::vector<int64_t> pos(h.tptr.begin(), h.tptr.end() - 1);
  for (int64_t d = 0; d < h.D; ++d)
    for (int64_t k = 0; k < h.fw[d]; ++k) {
      const int64_t i = h.flo[d] + k;
      h.tidx[pos[i]] = (int32_t)d;
      h.tval[pos[i]++] = h.fval[h.foff[d] + k];
    }
  h.bdiag.assign(h.M, 0.0);
  for (int64_t d = 0; d < h.D; ++d)
    for (int64_t k = 0; k < h.fw[d]; ++k) {
      const double f = h.fval[h.foff[d] + k];
      double& b = h.bdiag[h.flo[d] + k];
      b = b + 2.0 * (f * f);
    }
  if (h.gam != 0) {
    for (int64_t j = 0; j + 1 < h.M; ++j) h.bdiag[j] = h.bdiag[j] + 2.0 * h.gam;
    for (int64_t j = 1; j < h.M; ++j) h.bdiag[j] = h.bdiag[j] + 2.0 * h.gam;
  }
}

// Band form of F^T from the transposed CSR: row i spans d = tidx[first] ..
// tidx[last]; entries of d outside that row's CSR stay zero.
inline void transposed_bands(HostProblem& h) {
  h.tlo.assign(h.M, -1);
  h.tw.assign(h.M, 0);
  h.toff.assign(h.M, 0);
  int64_t tot = 0;
  for (int64_t i = 0; i < h.M; ++i) {
    h.toff[i] = tot;
    if (h.tptr[i + 1] > h.tptr[i]) {
      h.tlo[i] = h.tidx[h.tptr[i]];
      h.tw[i] = h.tidx[h.tptr[i + 1] - 1] - h.tlo[i] + 1;
      tot += h.tw[i];
    }
  }
  h.tbval.assign(tot, 0.0);
  for (int64_t i = 0; i < h.M; ++i)
    for (int64_t e = h.tptr[i]; e < h.tptr[i + 1]; ++e) h.tbval[h.toff[i] + h.tidx[e] - h.tlo[i]] = h.tval[e];
}

// Initial maxr from the seeded random X (pqdts.f90:1565-1575); call after P.
inline std::vector<int32_t> initial_maxr(int64_t M, int64_t N, SeededStream& rng) {
  std::vector<int32_t> mr(M);
  std::vector<double> row(N);
  for (int64_t i = 0; i < M; ++i) {
    double s = 0;
    for (int64_t n = 0; n < N; ++n) s += (row[n] = rng.next());
    int32_t am = 0;
    for (int64_t n = 0; n < N; ++n) {
      row[n] = row[n] / s;
      if (row[n] > row[am]) am = (int32_t)n;
    }
    mr[i] = am;
  }
  return mr;
}

}  // namespace pqdts
