// pqdts CPU ORACLE -- test infrastructure only.
//
// A C++17 restatement of the reference solver pc2/pqdts (pqdts.f90, single
// rank, no MPI) used by tests/ as the parity checker and by bench.py as the
// CPU baseline.  It is never linked into, called by, or shipped with the
// GPU product (pqdts_gb300/).  The product path fails loudly without its
// CUDA library instead of falling back to this code.
//
// Parity status: "parity unpinned" against the reference program itself.
// The reference is Fortran and no Fortran compiler exists on either build
// machine, so pqdts_omp.x cannot be run.  What IS pinned:
//   * the simplex projection (condat_project below) is bit-exact against the
//     reference's own condat_simplexproj.c, compiled from the reference tree
//     into oracle/_ref by oracle/build.py (tests/test_oracle.py);
//   * the derivative identities of the reference's built-in self test
//     (pqdts.f90:1737-1831) hold for L/dL/BF/Bdiag in full and reduced space
//     (tests/test_oracle.py).
//
// Arithmetic conventions (what makes this restatement deterministic):
//   * Reductions follow one fixed order of the reference: every Fortran
//     SUM(...) is a left-to-right chain; every OpenMP reduction is evaluated
//     as if each loop iteration ran on its own thread and the private sums
//     were combined in ascending order.  For pdot, L's residual sum and
//     conv_test this equals the single-thread order; for L's gamma term it
//     is the order of one thread per column (the reference's own value of
//     that term depends on OMP_NUM_THREADS).  OpenMP is used here only over
//     independent outputs, so the result does not depend on the thread
//     count.
//   * a + b*c in the Fortran source is evaluated as fma(b, c, a), the
//     contraction GCC applies under -O3 on FMA hardware; b*c + d*e keeps
//     the first product fused: fma(b, c, round(d*e)).
//   * Single-precision literals in the reference (1e-5, 1e-8, 1e-12, 1e-4)
//     are promoted from float, exactly as gfortran does.
//   * The reference's gfortran RANDOM_NUMBER stream (seed 23764) cannot be
//     reproduced without libgfortran; where the reference draws random
//     numbers (random P for nnzP<0, the initial random X that fixes the
//     first maxr) a splitmix64 stream seeded with 23764 is used instead.
//     The product implements the same stream so both agree.
//
// Layout follows the reference: X(M,N) column-major (X[i + n*M]), O(N,D)
// and P(N,D) column-major (O[n + d*N]).  Indices are 0-based; maxr = -1
// means "no max column" (the reference's full-space marker).

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// Reference constants (pqdts.f90), float literals promoted to double.
const double kDx = (double)1e-5f;          // Lalpha_min*: dx = 1e-5 (354, 404, 450)
const double kActiveTol = (double)1e-8f;   // tactivetol = 1e-8 (1207)
const double kFeasTol = (double)1e-12f;    // xmin .ge. -1e-12 (424, 430)
const double kStage1Exit = (double)1e-4f;  // abs(dlalpha) .lt. 1e-4 (1955)
const double kHuge = std::numeric_limits<double>::max();

double wtime() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------------------
// gfortran list-directed output (PRINT *, WRITE(u,*)) for the item kinds the
// reference prints: character, integer(4), integer(8), real(8).
// ---------------------------------------------------------------------------
struct LD {
  std::string s = " ";
  bool prev_char = true;  // the record's leading blank acts as separator
  bool first = true;
  LD& str(const std::string& t) {
    if (!first && !prev_char) s += ' ';
    s += t;
    prev_char = true;
    first = false;
    return *this;
  }
  void sep() {
    if (!first) s += ' ';
    first = false;
    prev_char = false;
  }
  LD& i4(long long v) {
    sep();
    char b[32];
    snprintf(b, sizeof b, "%11lld", v);
    s += b;
    return *this;
  }
  LD& i8(long long v) {
    sep();
    char b[32];
    snprintf(b, sizeof b, "%20lld", v);
    s += b;
    return *this;
  }
  LD& r8(double v) {
    sep();
    s += fmt_r8(v);
    return *this;
  }
  static std::string fmt_r8(double v) {
    char b[64];
    if (std::isnan(v)) {
      snprintf(b, sizeof b, "%25s", "NaN");
      return b;
    }
    if (std::isinf(v)) {
      snprintf(b, sizeof b, "%25s", v > 0 ? "Infinity" : "-Infinity");
      return b;
    }
    if (v == 0.0) {
      snprintf(b, sizeof b, "%20.16f     ", v);
      return b;
    }
    char e[64];
    snprintf(e, sizeof e, "%.16e", v);
    int ex = atoi(strchr(e, 'e') + 1);
    int k = ex + 1;  // 10^(k-1) <= |v| < 10^k after rounding to 17 digits
    if (k >= 0 && k <= 17) {
      snprintf(b, sizeof b, "%20.*f     ", 17 - k, v);
      return b;
    }
    std::string m(e, strchr(e, 'e'));
    char t[64];
    snprintf(t, sizeof t, "%sE%c%03d", m.c_str(), ex < 0 ? '-' : '+', ex < 0 ? -ex : ex);
    snprintf(b, sizeof b, "%25s", t);
    return b;
  }
  void print() const { printf("%s\n", s.c_str()); }
};

// ---------------------------------------------------------------------------
// Named wall-clock timers: tstart/tstop/tprint (pqdts.f90:103-186).
// ---------------------------------------------------------------------------
struct Timers {
  std::vector<std::string> name;
  std::vector<double> t0, sum;
  std::vector<int> cnt;
  bool opened = false;
  int find(const char* n) {
    for (size_t i = 0; i < name.size(); ++i)
      if (name[i] == n) return (int)i;
    return -1;
  }
  void start(const char* n) {
    int i = find(n);
    if (i < 0) {
      name.push_back(n);
      t0.push_back(0);
      sum.push_back(0);
      cnt.push_back(0);
      i = (int)name.size() - 1;
    }
    t0[i] = wtime();
    cnt[i]++;
  }
  void stop(const char* n) {
    int i = find(n);
    if (i < 0) return;
    sum[i] += wtime() - t0[i];
  }
  double total(const char* n) {
    int i = find(n);
    return i < 0 ? 0.0 : sum[i];
  }
  void print(int iter, const char* path) {
    // First call truncates when iter == 0 (or creates); later calls append.
    FILE* f = fopen(path, opened ? "a" : (iter == 0 ? "w" : "a"));
    opened = true;
    if (!f) return;
    for (size_t i = 0; i < name.size(); ++i) {
      char nm[32];
      snprintf(nm, sizeof nm, "%-20s", name[i].c_str());
      LD l;
      l.i4(iter).str(nm).i4(cnt[i]).r8(sum[i]);
      fprintf(f, "%s\n", l.s.c_str());
    }
    fclose(f);
  }
};

// splitmix64 stand-in for gfortran's RANDOM_NUMBER after set_seed (1109-1118).
struct SplitMix {
  uint64_t s;
  explicit SplitMix(uint64_t seed) : s(seed) {}
  double next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return (double)(z >> 11) * 0x1.0p-53;
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// Condat (2014) simplex projection, restated from the published algorithm
// (L. Condat, "Fast projection onto the simplex and the l1 ball", Math.
// Program. 158, 2016; preprint hal-01056171, Algorithm "proposed", a = 1).
// The visiting order of the published steps follows the reference's C code
// (condat_simplexproj.c:59-95): step 3 scans the deferred list from its end,
// step 4 scans the active list front to back, so rounding matches bit for bit.
// ---------------------------------------------------------------------------
extern "C" void orc_condat(const double* y, double* x, int64_t n) {
  if (n <= 0) return;
  std::vector<double> v, deferred, kept;
  v.reserve(n);
  v.push_back(y[0]);
  double rho = y[0] - 1.0;
  // Step 2: online filtering pass.
  for (int64_t i = 1; i < n; ++i) {
    if (y[i] > rho) {
      rho += (y[i] - rho) / (double)(v.size() + 1);
      if (rho > y[i] - 1.0) {
        v.push_back(y[i]);
      } else {
        deferred.insert(deferred.end(), v.begin(), v.end());
        v.clear();
        v.push_back(y[i]);
        rho = y[i] - 1.0;
      }
    }
  }
  // Step 3: re-admit deferred values above the threshold (scanned backwards,
  // each admitted value goes to the front of the active list).
  if (!deferred.empty()) {
    std::vector<double> front;
    for (size_t k = deferred.size(); k-- > 0;) {
      if (deferred[k] > rho) {
        front.push_back(deferred[k]);
        rho += (deferred[k] - rho) / (double)(v.size() + front.size());
      }
    }
    std::reverse(front.begin(), front.end());
    front.insert(front.end(), v.begin(), v.end());
    v.swap(front);
  }
  // Step 4: remove values below the threshold until the set is stable.
  for (;;) {
    size_t old = v.size();
    kept.clear();
    for (size_t k = 0; k < old; ++k) {
      if (v[k] > rho)
        kept.push_back(v[k]);
      else
        rho += (rho - v[k]) / (double)((old - 1 - k) + kept.size());
    }
    v.swap(kept);
    if (v.size() >= old) break;
  }
  for (int64_t i = 0; i < n; ++i) x[i] = y[i] > rho ? y[i] - rho : 0.0;
}

// ---------------------------------------------------------------------------
// Problem state: the module variables of `basics` (pqdts.f90:34-101).
// ---------------------------------------------------------------------------
struct Oracle {
  int64_t M = 0, N = 0, D = 0;
  double gam = 0;
  int mode = 2;
  bool tfullspace = true;
  int verbose = 0;  // print the reference's stdout lines
  // F as per-row dense bands (Flocalrow0/1 + Frows, 1318-1466), 0-based,
  // flo[d] = -1 for a row without entries.
  std::vector<int64_t> flo, fhi, foff;
  std::vector<double> fval;
  std::vector<double> P, O;  // (N,D) column-major
  std::vector<int32_t> maxr;
  std::vector<int8_t> ik;
  // work arrays of the main program (1540-1563)
  std::vector<double> Xtmp, sn, z, bd, dLdX;
  Timers t;

  size_t MN() const { return (size_t)M * (size_t)N; }
  double& x(std::vector<double>& a, int64_t i, int64_t n) { return a[i + n * M]; }

  // pqdts.f90:729 `sum(Frows(i)%f*X(lo:hi, j))`, 707-736 (local part).
  void redO(const double* X) {
    t.start("redO_O");
#pragma omp parallel for schedule(static)
    for (int64_t d = 0; d < D; ++d) {
      double* o = &O[(size_t)d * N];
      if (flo[d] < 0) {
        for (int64_t n = 0; n < N; ++n) o[n] = 0.0;
        continue;
      }
      const double* f = &fval[foff[d]];
      int64_t w = fhi[d] - flo[d] + 1;
      for (int64_t n = 0; n < N; ++n) {
        const double* xc = X + flo[d] + n * M;
        double s = 0.0;
        for (int64_t k = 0; k < w; ++k) s = std::fma(f[k], xc[k], s);
        o[n] = s;
      }
    }
    t.stop("redO_O");
  }

  // Row rebuild `X(j,maxr) = 1 - (sum(X(j,:)) - X(j,maxr))` (932, 987, 1048).
  void rebuild_max(double* X) {
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < M; ++j) {
      double s = 0.0;
      for (int64_t n = 0; n < N; ++n) s += X[j + n * M];
      double* xm = &X[j + (int64_t)maxr[j] * M];
      *xm = 1.0 - (s - *xm);
    }
  }

  // pqdts.f90:917-973
  double L(double* X) {
    t.start("L");
    if (!tfullspace) rebuild_max(X);
    redO(X);
    // L_red_calc: rows with a band only (946); chain over d, then 0 + chain.
    std::vector<double> rowsum(D, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t d = 0; d < D; ++d) {
      if (flo[d] < 0) continue;
      double s = 0.0;
      for (int64_t n = 0; n < N; ++n) {
        double r = O[(size_t)d * N + n] - P[(size_t)d * N + n];
        s = std::fma(r, r, s);
      }
      rowsum[d] = s;
    }
    double red = 0.0;
    for (int64_t d = 0; d < D; ++d)
      if (flo[d] >= 0) red = red + rowsum[d];
    double val = 0.0 + red;
    if (gam != 0) {
      // L_gam (956-962): `val = val + gam*(X(j,i)-X(j+1,i))**2` under
      // reduction(+:val) schedule(static,1) over columns i.  The reference's
      // result depends on OMP_NUM_THREADS here (the private accumulator of a
      // thread spans all its columns).  The oracle fixes the order of one
      // thread per column: a chain over rows per column, the columns' sums
      // then added to val in ascending column order.
      std::vector<double> colsum(N, 0.0);
#pragma omp parallel for schedule(static)
      for (int64_t n = 0; n < N; ++n) {
        const double* xc = X + n * M;
        double g = 0.0;
        for (int64_t j = 0; j + 1 < M; ++j) {
          double dx = xc[j] - xc[j + 1];
          g = std::fma(gam, dx * dx, g);
        }
        colsum[n] = g;
      }
      for (int64_t n = 0; n < N; ++n) val = val + colsum[n];
    }
    t.stop("L");
    return val;
  }

  // Gradient scatter `dLdX(band,j) += 2(O-P) F` (997-1006), chain over d.
  void scatter_T(double* G, const double* R2 /*(N,D): 2*(O-P) or 2*O*/) {
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      double* g = G + n * M;
      for (int64_t d = 0; d < D; ++d) {
        if (flo[d] < 0) continue;
        const double* f = &fval[foff[d]];
        double r = R2[(size_t)d * N + n];
        int64_t w = fhi[d] - flo[d] + 1;
        double* gb = g + flo[d];
        for (int64_t k = 0; k < w; ++k) gb[k] = std::fma(r, f[k], gb[k]);
      }
    }
  }

  // pqdts.f90:975-1032
  void dL(double* X, double* G) {
    t.start("dL");
    if (!tfullspace) rebuild_max(X);
    std::fill(G, G + MN(), 0.0);
    redO(X);
    std::vector<double> R2((size_t)D * N);
    for (size_t k = 0; k < R2.size(); ++k) R2[k] = 2.0 * (O[k] - P[k]);
    scatter_T(G, R2.data());
    if (gam != 0) {
      const double c = 2.0 * gam;
#pragma omp parallel for schedule(static)
      for (int64_t n = 0; n < N; ++n) {
        double* g = G + n * M;
        const double* xc = X + n * M;
        for (int64_t j = 0; j < M; ++j) {
          if (j < M - 1) g[j] = std::fma(c, xc[j] - xc[j + 1], g[j]);
          if (j > 0) g[j] = std::fma(-c, xc[j - 1] - xc[j], g[j]);
        }
      }
    }
    if (!tfullspace) {
#pragma omp parallel for schedule(static)
      for (int64_t j = 0; j < M; ++j) {
        double gm = G[j + (int64_t)maxr[j] * M];
        for (int64_t n = 0; n < N; ++n) G[j + n * M] = G[j + n * M] - gm;
      }
    }
    t.stop("dL");
  }

  // pqdts.f90:208-244 (the value is the same for every column n).
  void Bdiag(double* BD) {
    t.start("Bdiag");
    std::vector<double> col(M, 0.0);
    for (int64_t d = 0; d < D; ++d) {
      if (flo[d] < 0) continue;
      const double* f = &fval[foff[d]];
      int64_t w = fhi[d] - flo[d] + 1;
      for (int64_t k = 0; k < w; ++k) col[flo[d] + k] = col[flo[d] + k] + 2.0 * (f[k] * f[k]);
    }
    if (gam != 0) {
      for (int64_t j = 0; j < M - 1; ++j) col[j] = col[j] + 2.0 * gam;
      for (int64_t j = 1; j < M; ++j) col[j] = col[j] + 2.0 * gam;
    }
    if (!tfullspace)
      for (int64_t j = 0; j < M; ++j) col[j] = col[j] * 2.0;
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < N; ++n) std::copy(col.begin(), col.end(), BD + n * M);
    t.stop("Bdiag");
  }

  // Row sum of dd without the max column: sum(dd(j,:)) - dd(j,maxr(j)).
  double rest(const double* dd, int64_t j) {
    double s = 0.0;
    for (int64_t n = 0; n < N; ++n) s += dd[j + n * M];
    return s - dd[j + (int64_t)maxr[j] * M];
  }

  // pqdts.f90:246-342  BX = H * dd
  void BF(const double* dd, double* BX) {
    t.start("BF");
    std::vector<double> rs;
    if (!tfullspace) {
      rs.resize(M);
      for (int64_t j = 0; j < M; ++j) rs[j] = rest(dd, j);
      std::copy(dd, dd + MN(), BX);
      for (int64_t j = 0; j < M; ++j) BX[j + (int64_t)maxr[j] * M] = -rs[j];
      redO(BX);
    } else {
      redO(dd);
    }
    std::fill(BX, BX + MN(), 0.0);
    std::vector<double> R2((size_t)D * N);
    for (size_t k = 0; k < R2.size(); ++k) R2[k] = 2.0 * O[k];
    // 2.0*f*O == fma(2f, O, .) == fma(2O, f, .): the factor 2 is exact.
    scatter_T(BX, R2.data());
    if (gam != 0) {
      const double c = 2.0 * gam;
#pragma omp parallel for schedule(static)
      for (int64_t n = 0; n < N; ++n) {
        double* b = BX + n * M;
        const double* v = dd + n * M;
        for (int64_t j = 0; j < M; ++j) {
          if (j < M - 1) {
            b[j] = std::fma(c, v[j] - v[j + 1], b[j]);
            if (!tfullspace) {
              if (n == maxr[j]) b[j] = std::fma(c, -v[j] - rs[j], b[j]);
              if (n == maxr[j + 1]) b[j] = std::fma(c, v[j + 1] + rs[j + 1], b[j]);
            }
          }
          if (j > 0) {
            b[j] = std::fma(-c, v[j - 1] - v[j], b[j]);
            if (!tfullspace) {
              if (n == maxr[j - 1]) b[j] = std::fma(-c, -v[j - 1] - rs[j - 1], b[j]);
              if (n == maxr[j]) b[j] = std::fma(-c, v[j] + rs[j], b[j]);
            }
          }
        }
      }
    }
    if (!tfullspace) {
      for (int64_t j = 0; j < M; ++j) {
        double bm = BX[j + (int64_t)maxr[j] * M];
        for (int64_t n = 0; n < N; ++n) BX[j + n * M] = BX[j + n * M] - bm;
      }
    }
    t.stop("BF");
  }

  // pdot (589-614): 0 + chain over columns of per-column chains.
  double pdot(const double* a, const double* b) {
    std::vector<double> cs(N);
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < N; ++n) {
      double s = 0.0;
      for (int64_t j = 0; j < M; ++j) s = std::fma(a[j + n * M], b[j + n * M], s);
      cs[n] = s;
    }
    double v = 0.0;
    for (int64_t n = 0; n < N; ++n) v = v + cs[n];
    return 0.0 + v;
  }

  // doproj (1120-1140)
  void doproj(double* X) {
    t.start("doproj");
#pragma omp parallel
    {
      std::vector<double> x3(N), x2(N);
#pragma omp for schedule(static)
      for (int64_t i = 0; i < M; ++i) {
        for (int64_t n = 0; n < N; ++n) x3[n] = X[i + n * M];
        orc_condat(x3.data(), x2.data(), N);
        for (int64_t n = 0; n < N; ++n) X[i + n * M] = x2[n];
      }
    }
    t.stop("doproj");
  }

  // doproj2 (1142-1164)
  double doproj2(double* X) {
    t.start("doproj2");
    double xmin = 0.0;
    for (int64_t i = 0; i < M; ++i) {
      for (int64_t n = 0; n < N; ++n)
        if (X[i + n * M] < 0) X[i + n * M] = 0.0;
      double s = 0.0;
      for (int64_t n = 0; n < N; ++n) s += X[i + n * M];
      double* xm = &X[i + (int64_t)maxr[i] * M];
      *xm = 1.0 - (s - *xm);
      xmin = std::min(xmin, *xm);
    }
    t.stop("doproj2");
    return xmin;
  }

  // conv_test (1034-1067)
  double conv_test(double* X, double* G, bool tprint) {
    if (!tfullspace) rebuild_max(X);
    tfullspace = true;
    dL(X, G);
    double conv = 0.0;
    for (int64_t i = 0; i < M; ++i) {
      double mn = kHuge;
      for (int64_t n = 0; n < N; ++n) mn = std::min(mn, G[i + n * M]);
      double lambda = std::max(0.0, -mn);
      double s = 0.0;
      for (int64_t n = 0; n < N; ++n) {
        double tt = (G[i + n * M] + lambda) * X[i + n * M];
        s = std::fma(tt, tt, s);
      }
      conv = conv + s;
      if (tprint && verbose) {
        double m2 = kHuge;
        for (int64_t n = 0; n < N; ++n) m2 = std::min(m2, G[i + n * M] + lambda);
        LD l;
        l.str("lambda").i8(i + 1).r8(lambda).r8(m2).print();
      }
    }
    conv = 0.0 + conv;
    return std::sqrt(conv / ((double)N * (double)M));
  }

  // z = beta*y + alpha*x  (pgaxpy2 515-528) with the first product fused.
  void pgaxpy2(double alpha, const double* xv, double beta, const double* y, double* zv) {
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < (int64_t)MN(); ++k) zv[k] = std::fma(beta, y[k], alpha * xv[k]);
  }

  // Lalpha_min_auglag (440-483) and Lalpha_min2 (394-438).
  void line_search(double* X, const double* S, bool stage2, double& alpha, double& dlalpha) {
    t.start("Lalpha_min");
    double xmin = 0;
    alpha = 0.0;
    pgaxpy2(1.0, X, alpha, S, Xtmp.data());
    if (stage2) xmin = doproj2(Xtmp.data()); else doproj(Xtmp.data());
    double L0 = L(Xtmp.data());
    pgaxpy2(1.0, X, alpha + kDx, S, Xtmp.data());
    if (stage2) xmin = doproj2(Xtmp.data()); else doproj(Xtmp.data());
    double Lp = L(Xtmp.data());
    double df = (Lp - L0) / kDx;
    dlalpha = df;
    alpha = 1.0;
    double lm = kHuge, alphamin = 0;
    for (int i = 1; i <= 100; ++i) {
      pgaxpy2(1.0, X, alpha, S, Xtmp.data());
      if (stage2) xmin = doproj2(Xtmp.data()); else doproj(Xtmp.data());
      Lp = L(Xtmp.data());
      bool ok = stage2 ? (Lp < lm && xmin >= -kFeasTol) : (Lp < lm);
      if (ok) {
        lm = Lp;
        alphamin = alpha;
      }
      if (verbose) {
        LD l;
        l.str("line search").i8(i).str("L=").r8(Lp).str("alpha=").r8(alpha).str("df(0)=").r8(df);
        if (stage2) l.str("min(X)=").r8(xmin);
        l.print();
      }
      double armijo = std::fma(0.1 * alpha, df, L0);
      bool shrink = stage2 ? (Lp > armijo || xmin < -kFeasTol) : (Lp > armijo);
      if (shrink) alpha = alpha * 0.75;
      else break;
    }
    alpha = alphamin;
    t.stop("Lalpha_min");
  }
};

// Reference band build from COO (1318-1365): band = [min col, max col] of the
// row, zero filled, later duplicates overwrite earlier ones (1361).
static void build_bands_coo(Oracle& o, int64_t nnz, const int32_t* row, const int32_t* col, const double* val) {
  int64_t D = o.D;
  o.flo.assign(D, -1);
  o.fhi.assign(D, -1);
  for (int64_t k = 0; k < nnz; ++k) {
    int64_t d = row[k], i = col[k];
    if (o.flo[d] < 0 || i < o.flo[d]) o.flo[d] = i;
    if (i > o.fhi[d]) o.fhi[d] = i;
  }
  o.foff.assign(D, 0);
  int64_t tot = 0;
  for (int64_t d = 0; d < D; ++d) {
    o.foff[d] = tot;
    if (o.flo[d] >= 0) tot += o.fhi[d] - o.flo[d] + 1;
  }
  o.fval.assign(tot, 0.0);
  for (int64_t k = 0; k < nnz; ++k) {
    int64_t d = row[k];
    o.fval[o.foff[d] + col[k] - o.flo[d]] = val[k];
  }
}

// fprob (188-206)
static double fprob(double x, double mean) {
  const double pi = 4.0 * std::atan(1.0);
  if (mean < 50) {
    if (mean == 0 && x == 0) return 1.0;
    double lf = std::lgamma(x + 1.0);
    return std::exp(std::fma(std::log(mean), x, -lf) - mean);
  }
  double y = (x - mean) / std::sqrt(mean);
  return std::exp(-0.5 * (y * y)) / std::sqrt(mean) / std::sqrt(2 * pi);
}

// Internal F (1366-1466), single rank: needs M == (D-1)^2.
static int build_bands_internal(Oracle& o) {
  int64_t D = o.D, M = o.M;
  if (M != (D - 1) * (D - 1)) return -1;
  o.flo.assign(D, -1);
  o.fhi.assign(D, -1);
  for (int64_t i = 1; i <= D; ++i) {
    int64_t mean = (D - i) * (D - i);
    int64_t i0 = std::numeric_limits<int64_t>::max(), i1 = 0;
    for (int64_t j = std::max<int64_t>(1, mean); j <= M; ++j) {
      if (fprob((double)(j - 1), (double)mean) < 1e-10) break;
      i0 = std::min(j, i0);
      i1 = std::max(j, i1);
    }
    for (int64_t j = std::max<int64_t>(1, mean); j >= 1; --j) {
      if (fprob((double)(j - 1), (double)mean) < 1e-10) break;
      i0 = std::min(j, i0);
      i1 = std::max(j, i1);
    }
    if (i1 >= 1 && i0 <= M) {
      o.flo[i - 1] = i0 - 1;
      o.fhi[i - 1] = i1 - 1;
    }
  }
  o.foff.assign(D, 0);
  int64_t tot = 0;
  for (int64_t d = 0; d < D; ++d) {
    o.foff[d] = tot;
    if (o.flo[d] >= 0) tot += o.fhi[d] - o.flo[d] + 1;
  }
  o.fval.assign(tot, 0.0);
  for (int64_t d = 0; d < D; ++d) {
    if (o.flo[d] < 0) continue;
    int64_t mean = (D - (d + 1)) * (D - (d + 1));
    for (int64_t j = o.flo[d]; j <= o.fhi[d]; ++j) o.fval[o.foff[d] + j - o.flo[d]] = fprob((double)j, (double)mean);
  }
  return 0;
}

// ---------------------------------------------------------------------------
// C ABI used by the tests (ctypes) and by the CLI below.
// ---------------------------------------------------------------------------
extern "C" {

void* orc_create(int64_t M, int64_t N, int64_t D, double gam, int64_t nnzF, const int32_t* Frow, const int32_t* Fcol,
                 const double* Fval, int64_t nnzP, const int32_t* Prow, const int32_t* Pcol, const double* Pval) {
  Oracle* o = new Oracle();
  o->M = M;
  o->N = N;
  o->D = D;
  o->gam = gam;
  if (nnzF >= 0) {
    for (int64_t k = 0; k < nnzF; ++k)
      if (Frow[k] < 0 || Frow[k] >= D || Fcol[k] < 0 || Fcol[k] >= M) {
        delete o;
        return nullptr;
      }
    build_bands_coo(*o, nnzF, Frow, Fcol, Fval);
  } else if (build_bands_internal(*o) != 0) {
    delete o;
    return nullptr;
  }
  SplitMix rng(23764);
  o->P.assign((size_t)N * D, 0.0);
  if (nnzP >= 0) {
    for (int64_t k = 0; k < nnzP; ++k) {
      if (Prow[k] < 0 || Prow[k] >= D || Pcol[k] < 0 || Pcol[k] >= N) {
        delete o;
        return nullptr;
      }
      o->P[(size_t)Prow[k] * N + Pcol[k]] = Pval[k];
    }
  } else {
    for (size_t k = 0; k < o->P.size(); ++k) o->P[k] = rng.next();
  }
  o->O.assign((size_t)N * D, 0.0);
  size_t mn = o->MN();
  o->Xtmp.assign(mn, 0.0);
  o->sn.assign(mn, 0.0);
  o->z.assign(mn, 0.0);
  o->bd.assign(mn, 0.0);
  o->dLdX.assign(mn, 0.0);
  o->ik.assign(mn, 0);
  // Initial maxr from a random feasible X (1565-1575).
  o->maxr.assign(M, 0);
  std::vector<double> row(N);
  for (int64_t i = 0; i < M; ++i) {
    double s = 0;
    for (int64_t n = 0; n < N; ++n) s += (row[n] = rng.next());
    int32_t am = 0;
    for (int64_t n = 0; n < N; ++n) {
      row[n] = row[n] / s;
      if (row[n] > row[am]) am = (int32_t)n;
    }
    o->maxr[i] = am;
  }
  return o;
}

void orc_destroy(void* h) { delete (Oracle*)h; }

void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

int64_t orc_band(void* h, int64_t* lo, int64_t* hi, int64_t* off) {
  Oracle* o = (Oracle*)h;
  for (int64_t d = 0; d < o->D; ++d) {
    if (lo) lo[d] = o->flo[d];
    if (hi) hi[d] = o->fhi[d];
    if (off) off[d] = o->foff[d];
  }
  return (int64_t)o->fval.size();
}

void orc_band_values(void* h, double* vals) {
  Oracle* o = (Oracle*)h;
  std::copy(o->fval.begin(), o->fval.end(), vals);
}

void orc_get_P(void* h, double* P) {
  Oracle* o = (Oracle*)h;
  std::copy(o->P.begin(), o->P.end(), P);
}

void orc_set_space(void* h, int fullspace, const int32_t* maxr) {
  Oracle* o = (Oracle*)h;
  o->tfullspace = fullspace != 0;
  if (maxr) std::copy(maxr, maxr + o->M, o->maxr.begin());
}

void orc_get_maxr(void* h, int32_t* maxr) {
  Oracle* o = (Oracle*)h;
  std::copy(o->maxr.begin(), o->maxr.end(), maxr);
}

double orc_L(void* h, double* X) { return ((Oracle*)h)->L(X); }
void orc_redO(void* h, const double* X, double* O) {
  Oracle* o = (Oracle*)h;
  o->redO(X);
  std::copy(o->O.begin(), o->O.end(), O);
}
void orc_dL(void* h, double* X, double* G) { ((Oracle*)h)->dL(X, G); }
void orc_BF(void* h, const double* dd, double* BX) { ((Oracle*)h)->BF(dd, BX); }
void orc_Bdiag(void* h, double* BD) { ((Oracle*)h)->Bdiag(BD); }
void orc_doproj(void* h, double* X) { ((Oracle*)h)->doproj(X); }
double orc_doproj2(void* h, double* X) { return ((Oracle*)h)->doproj2(X); }
double orc_conv_test(void* h, double* X, double* G) { return ((Oracle*)h)->conv_test(X, G, false); }
double orc_pdot(void* h, const double* a, const double* b) { return ((Oracle*)h)->pdot(a, b); }
double orc_timer(void* h, const char* name) { return ((Oracle*)h)->t.total(name); }

// The stage loop of `program pqdts` from the first objective (1908) to the
// end of the last stage (2167), modes 1 and 2.  X (M,N) column-major is the
// starting point and receives the result.  stats[0..7] = final L, conv,
// ||der||, outer iterations, CG iterations, line-search probes, dL calls,
// seconds in the `min` timer.  stage_cb (may be null) runs after each stage.
int orc_solve(void* h, double* X, int mode, int maxiiter, double conv_thres, int start_stage, int output, int verbose,
              double* stats, void (*stage_cb)(void*, int, const double*), void* cb_user) {
  Oracle& o = *(Oracle*)h;
  o.mode = mode;
  o.verbose = verbose;
  const int64_t M = o.M, N = o.N;
  const size_t mn = o.MN();
  double* dLdX = o.dLdX.data();
  double* sn = o.sn.data();
  double* z = o.z.data();
  double* bd = o.bd.data();
  double* xtmp = o.Xtmp.data();
  int64_t n_outer = 0, n_cg = 0, n_ls0 = 0;
  double L0 = o.L(X);
  o.dL(X, dLdX);
  double norm_der = o.pdot(dLdX, dLdX);
  if (verbose) {
    LD l;
    l.str("iter").i4(0).i4(0).str("L=").r8(L0).str("||der||=").r8(std::sqrt(norm_der)).str("dt=").r8(0.0).str("ttot=").r8(0.0);
    l.print();
  }
  double t0 = wtime();
  o.t.start("min");
  double conv = 0, alpha = 0, xmin = 0, dlalpha = kHuge;
  for (int oiter = start_stage; oiter <= 2; ++oiter) {
    dlalpha = -kHuge;
    for (int iiter = 1; iiter <= maxiiter; ++iiter) {
      double t1 = wtime();
      if (mode == 1) {
        o.tfullspace = false;
        for (int64_t j = 0; j < M; ++j) {
          int32_t am = 0;
          for (int64_t n = 1; n < N; ++n)
            if (X[j + n * M] > X[j + (int64_t)am * M]) am = (int32_t)n;
          o.maxr[j] = am;
          X[j + (int64_t)am * M] = 1.0;
        }
        o.dL(X, dLdX);
        for (size_t k = 0; k < mn; ++k) sn[k] = dLdX[k] * -1.0;
        o.line_search(X, sn, true, alpha, dlalpha);
      } else {
        if ((std::fabs(dlalpha) < kStage1Exit || dlalpha > 0) && oiter == 1) {
          if (verbose) {
            LD l;
            l.str("stopping inner iteration because dldlpha is small").r8(dlalpha).print();
          }
          break;
        }
        o.tfullspace = (oiter == 1);
        if (!o.tfullspace) {
          for (int64_t j = 0; j < M; ++j) {
            if (o.maxr[j] != -1) {
              double s = 0.0;
              for (int64_t n = 0; n < N; ++n) s += X[j + n * M];
              double* xm = &X[j + (int64_t)o.maxr[j] * M];
              *xm = 1.0 - (s - *xm);
            }
            int32_t am = 0;
            for (int64_t n = 1; n < N; ++n)
              if (X[j + n * M] > X[j + (int64_t)am * M]) am = (int32_t)n;
            o.maxr[j] = am;
            X[j + (int64_t)am * M] = 1.0;
          }
        } else {
          std::fill(o.maxr.begin(), o.maxr.end(), -1);
        }
        o.dL(X, dLdX);
        // active set (1986-2005)
        int64_t nact = 0;
        for (size_t k = 0; k < mn; ++k) {
          if (X[k] < kActiveTol && dLdX[k] > 0) {
            dLdX[k] = 0;
            o.ik[k] = 1;
            nact++;
          } else {
            o.ik[k] = 0;
          }
        }
        if (verbose) {
          LD l;
          l.str("positivity constraints").i8(nact).str("active of").i8(M * N).r8((double)nact / (double)(M * N)).print();
        }
        norm_der = o.pdot(dLdX, dLdX);
        std::fill(sn, sn + mn, 0.0);
        std::fill(z, z + mn, 0.0);
        for (size_t k = 0; k < mn; ++k) dLdX[k] = dLdX[k] * -1.0;  // r = -g
        o.Bdiag(bd);
        for (size_t k = 0; k < mn; ++k) z[k] = dLdX[k] / std::sqrt(bd[k]);
        double eps = std::min(0.5, std::sqrt(std::sqrt(norm_der))) * std::sqrt(norm_der);
        std::copy(z, z + mn, xtmp);
        for (int j = 1; j <= 50; ++j) {
          o.BF(xtmp, bd);
          n_cg++;
          for (size_t k = 0; k < mn; ++k)
            if (o.ik[k] == 1) bd[k] = 0;
          double b1 = o.pdot(dLdX, z);
          double v2 = o.pdot(xtmp, bd);
          double a1 = b1 / v2, a2 = -b1 / v2;
          for (size_t k = 0; k < mn; ++k) sn[k] = std::fma(a1, xtmp[k], sn[k]);
          for (size_t k = 0; k < mn; ++k) dLdX[k] = std::fma(a2, bd[k], dLdX[k]);
          o.Bdiag(bd);
          for (size_t k = 0; k < mn; ++k) z[k] = dLdX[k] / std::sqrt(bd[k]);
          v2 = o.pdot(dLdX, z);
          double beta = v2 / b1;
          for (size_t k = 0; k < mn; ++k) xtmp[k] = std::fma(beta, xtmp[k], 1.0 * z[k]);
          double b2 = o.pdot(dLdX, dLdX);
          if (verbose) {
            LD l;
            l.str("newton-pcg").i4(j).str("sqrt(b2)=").r8(std::sqrt(b2)).str("eps=").r8(eps).str("b1=").r8(b1).str("v2=").r8(v2);
            l.print();
          }
          if (std::sqrt(b2) <= eps) break;
        }
        o.dL(X, dLdX);
        o.Bdiag(bd);
        for (int64_t i = 0; i < N; ++i)
          for (int64_t k = 0; k < M; ++k)
            if (o.ik[k + i * M] == 1 && o.maxr[k] != i) sn[k + i * M] = -dLdX[k + i * M] / bd[k + i * M];
        o.line_search(X, sn, !o.tfullspace, alpha, dlalpha);
      }
      n_ls0++;
      if (alpha != 0)
        for (size_t k = 0; k < mn; ++k) X[k] = std::fma(alpha, sn[k], X[k]);
      xmin = 0;
      if (o.tfullspace) o.doproj(X);
      else xmin = o.doproj2(X);
      L0 = o.L(X);
      o.dL(X, dLdX);
      norm_der = o.pdot(dLdX, dLdX);
      conv = o.conv_test(X, dLdX, false);
      n_outer++;
      double t2 = wtime();
      if (verbose) {
        LD l;
        l.str("iter").i4(oiter).i4(iiter).str("L=").r8(L0).str("max(abs(c))").r8(xmin).str("conv").r8(conv);
        l.str("||der||=").r8(std::sqrt(norm_der)).str("mode=").i4(mode).str("alpha=").r8(alpha).str("dlalpha=").r8(dlalpha);
        l.str("dt=").r8(t2 - t1).str("ttot=").r8(t2 - t0);
        l.print();
      }
      if (conv < conv_thres) break;
    }
    conv = o.conv_test(X, dLdX, output >= 3);
    if (stage_cb) stage_cb(cb_user, oiter, X);
  }
  o.t.stop("min");
  if (stats) {
    stats[0] = L0;
    stats[1] = conv;
    stats[2] = std::sqrt(norm_der);
    stats[3] = (double)n_outer;
    stats[4] = (double)n_cg;
    stats[5] = (double)n_ls0;
    stats[6] = 0;
    stats[7] = o.t.total("min");
  }
  return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// CLI: identical arguments, inputs and outputs to pqdts_omp.x (1191-2231).
// ---------------------------------------------------------------------------
namespace {

bool read_raw(const char* path, void* buf, size_t bytes) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  size_t got = fread(buf, 1, bytes, f);
  fclose(f);
  return got == bytes;
}

// gfortran sequential unformatted record (4-byte markers, subrecords > 2^31-9 B).
void write_record(FILE* f, const void* data, size_t bytes) {
  const size_t kMax = 2147483639u;
  const char* p = (const char*)data;
  size_t left = bytes;
  bool first = true;
  do {
    size_t chunk = std::min(left, kMax);
    bool more = left > chunk;
    int32_t lead = (int32_t)chunk, tail = (int32_t)chunk;
    if (more) lead = -lead;
    if (!first) tail = -tail;
    fwrite(&lead, 4, 1, f);
    fwrite(p, 1, chunk, f);
    fwrite(&tail, 4, 1, f);
    p += chunk;
    left -= chunk;
    first = false;
  } while (left > 0);
}

bool read_record(FILE* f, std::vector<char>& out) {
  out.clear();
  for (;;) {
    int32_t lead, tail;
    if (fread(&lead, 4, 1, f) != 1) return false;
    size_t len = (size_t)(lead < 0 ? -(int64_t)lead : lead);
    size_t at = out.size();
    out.resize(at + len);
    if (len && fread(out.data() + at, 1, len, f) != len) return false;
    if (fread(&tail, 4, 1, f) != 1) return false;
    if (lead >= 0) return true;
  }
}

void write_state(const char* path, int64_t M, int64_t N, int64_t D, int32_t rank, const double* X) {
  FILE* f = fopen(path, "wb");
  if (!f) return;
  write_record(f, &M, 8);
  write_record(f, &N, 8);
  write_record(f, &D, 8);
  write_record(f, &M, 8);  // localrows
  write_record(f, &rank, 4);
  write_record(f, X, (size_t)M * N * 8);
  fclose(f);
}

void write_status() {
  FILE* in = fopen("/proc/self/status", "r");
  FILE* out = fopen("status_           0 .out", "w");
  if (!in || !out) {
    if (in) fclose(in);
    if (out) fclose(out);
    return;
  }
  char line[4096];
  while (fgets(line, sizeof line, in)) {
    char a[2048] = {0}, b[2048] = {0};
    if (sscanf(line, "%2047s %2047[^ \t\n,]", a, b) < 1) continue;
    fprintf(out, " %s %s\n", a, b);
  }
  fclose(in);
  fclose(out);
}

struct CbCtx {
  Oracle* o;
  int output;
};

void stage_file(void* u, int oiter, const double* X) {
  CbCtx* c = (CbCtx*)u;
  if (c->output >= 2) {
    char name[64];
    snprintf(name, sizeof name, "rank_%6d_oiter%6d.dat", 0, oiter);
    printf(" %s\n", name);
    c->o->t.start("output");
    write_state(name, c->o->M, c->o->N, c->o->D, 0, X);
    c->o->t.stop("output");
  }
  c->o->t.print(oiter, "timing_           0 .out");
}

}  // namespace

extern "C" int orc_main(int argc, char** argv) {
  if (argc < 15) {
    fprintf(stderr, "usage: %s M N D nnzF nnzP mode maxiter output gamma eps start_stage read_input smo_fact bench\n",
            argv[0]);
    return 1;
  }
  int64_t M = atoll(argv[1]), N = atoll(argv[2]), D = atoll(argv[3]);
  int64_t Fl = atoll(argv[4]), Pl = atoll(argv[5]);
  int mode = atoi(argv[6]), maxiiter = atoi(argv[7]), output = atoi(argv[8]);
  double gam = atof(argv[9]), conv_thres = atof(argv[10]);
  int start_stage = atoi(argv[11]), read_input = atoi(argv[12]);
  double smo_fact = atof(argv[13]);
  double t_prep0 = wtime();
  {
    LD l;
    l.str("num_proc").i4(1).print();
  }
  std::vector<int32_t> Fr, Fc, Pr, Pc;
  std::vector<double> Fv, Pv;
  if (Fl >= 0) {
    Fr.resize(Fl);
    Fc.resize(Fl);
    Fv.resize(Fl);
    if (!read_raw("data/F_row.bin", Fr.data(), Fl * 4) || !read_raw("data/F_col.bin", Fc.data(), Fl * 4) ||
        !read_raw("data/F_data.bin", Fv.data(), Fl * 8)) {
      LD l;
      l.str("cannot read data/F_*.bin").print();
      return 1;
    }
  }
  if (Pl >= 0) {
    Pr.resize(Pl);
    Pc.resize(Pl);
    Pv.resize(Pl);
    if (!read_raw("data/P_row.bin", Pr.data(), Pl * 4) || !read_raw("data/P_col.bin", Pc.data(), Pl * 4) ||
        !read_raw("data/P_data.bin", Pv.data(), Pl * 8)) {
      LD l;
      l.str("cannot read data/P_*.bin").print();
      return 1;
    }
  }
  if (Fl < 0 && M != (D - 1) * (D - 1)) {
    LD l;
    l.str("M is not (D-1)**2").print();
    return 0;
  }
  Oracle* o = (Oracle*)orc_create(M, N, D, gam, Fl, Fr.data(), Fc.data(), Fv.data(), Pl, Pr.data(), Pc.data(), Pv.data());
  if (!o) {
    LD l;
    l.str("invalid F or P input").print();
    return 1;
  }
  o->t.start("prep");
  std::vector<double> X((size_t)M * N, 1.0 / (double)N);
  if (read_input == 1) {
    FILE* f = fopen("data/initial_     0.dat", "rb");
    if (f) {
      LD l;
      l.str("reading starting state from").str("data/initial_     0.dat").print();
      std::vector<char> r;
      int64_t h[4];
      for (int k = 0; k < 4; ++k) {
        if (!read_record(f, r) || r.size() < 8) return 1;
        memcpy(&h[k], r.data(), 8);
      }
      if (!read_record(f, r) || r.size() < 4) return 1;
      int32_t rank2;
      memcpy(&rank2, r.data(), 4);
      const char* what[4] = {"M", "N", "D", "localrows"};
      int64_t want[4] = {M, N, D, M};
      for (int k = 0; k < 4; ++k)
        if (h[k] != want[k]) {
          LD l2;
          l2.str("input file in this directory is for a different").str(what[k]).i8(want[k]).str("!=").i8(h[k]).print();
          return 0;
        }
      if (rank2 != 0) return 0;
      if (!read_record(f, r) || r.size() < X.size() * 8) return 1;
      memcpy(X.data(), r.data(), X.size() * 8);
      fclose(f);
      if (smo_fact > 0) {  // smoothing (1877-1902)
        std::vector<double> Y(X);
        for (int64_t j = 1; j <= M; ++j) {
          if (j <= 100) continue;
          int64_t dist = (int64_t)std::llround((double)j / smo_fact);
          for (int64_t i = 0; i < N; ++i) {
            double s = 0;
            int64_t c = 0;
            for (int64_t k = std::max<int64_t>(1, j - dist); k <= std::min(j + dist, M); ++k) {
              s = s + X[(k - 1) + i * M];
              c++;
            }
            Y[(j - 1) + i * M] = s / (double)c;
          }
          double rs = 0;
          for (int64_t i = 0; i < N; ++i) rs += Y[(j - 1) + i * M];
          for (int64_t i = 0; i < N; ++i) Y[(j - 1) + i * M] = Y[(j - 1) + i * M] / rs;
        }
        X.swap(Y);
      }
    }
  }
  o->t.stop("prep");
  (void)t_prep0;
  o->t.print(0, "timing_           0 .out");
  CbCtx cb{o, output};
  double stats[8];
  orc_solve(o, X.data(), mode, maxiiter, conv_thres, start_stage, output, 1, stats, stage_file, &cb);
  if (output >= 1) {
    printf(" %s\n", "rank_     0_final.dat");
    o->t.start("output");
    write_state("rank_     0_final.dat", M, N, D, 0, X.data());
    o->t.stop("output");
  }
  o->t.print(-1, "timing_           0 .out");
  write_status();
  orc_destroy(o);
  return 0;
}

#ifdef ORACLE_MAIN
int main(int argc, char** argv) { return orc_main(argc, argv); }
#endif
