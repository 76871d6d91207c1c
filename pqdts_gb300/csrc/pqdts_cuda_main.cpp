// pqdts_cuda.x -- command-line drop-in for pqdts_omp.x (pqdts.f90:1191-2231).
//
//   pqdts_cuda.x M N D nnzF nnzP mode maxiter output gamma eps start_stage
//                read_input smo_fact bench
//
// Same positional arguments (1243-1270), same inputs in ./data/
// (F_/P_{row,col,data}.bin, initial_     0.dat), same outputs in the working
// directory (rank_     0_oiter     k.dat, rank_     0_final.dat,
// timing_           0 .out, status_           0 .out) and the same stdout
// lines, so pqdts.py drives it unchanged through `-p pqdts_cuda.x`.
// The solve itself runs in libpqdts_cuda.so on GPU 0 (PQDTS_DEVICE selects
// another); PQDTS_PRECISION=mixed selects the mixed-precision solver.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pqdts_cuda.h"
#include "fortran_io.h"

using pqdts::ListLine;

namespace {

double wall() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

bool read_raw(const char* path, void* buf, size_t bytes) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  size_t got = bytes ? fread(buf, 1, bytes, f) : 0;
  fclose(f);
  return got == bytes;
}

// Host timers with the reference's file format (tstart/tstop/tprint).
struct HostTimers {
  std::vector<std::string> names;
  std::vector<double> t0, sum;
  std::vector<int> cnt;
  bool opened = false;
  int id(const char* n) {
    for (size_t i = 0; i < names.size(); ++i)
      if (names[i] == n) return (int)i;
    names.push_back(n);
    t0.push_back(0);
    sum.push_back(0);
    cnt.push_back(0);
    return (int)names.size() - 1;
  }
  void start(const char* n) {
    int i = id(n);
    t0[i] = wall();
    cnt[i]++;
  }
  void stop(const char* n) {
    int i = id(n);
    sum[i] += wall() - t0[i];
  }
  void set(const char* n, double secs, long long count) {
    int i = id(n);
    sum[i] = secs;
    cnt[i] = (int)count;
  }
  void print(int iter) {
    const std::string path = pqdts::listed_file_name("timing_", 0);
    FILE* f = fopen(path.c_str(), opened ? "a" : (iter == 0 ? "w" : "a"));
    opened = true;
    if (!f) return;
    for (size_t i = 0; i < names.size(); ++i) {
      char nm[32];
      snprintf(nm, sizeof nm, "%-20s", names[i].c_str());
      ListLine l;
      l.i4(iter).s(nm).i4(cnt[i]).r8(sum[i]);
      fprintf(f, "%s\n", l.str().c_str());
    }
    fclose(f);
  }
};

void write_status() {
  FILE* in = fopen("/proc/self/status", "r");
  const std::string path = pqdts::listed_file_name("status_", 0);
  FILE* out = fopen(path.c_str(), "w");
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

struct StageCtx {
  int64_t M, N, D;
  int output;
  HostTimers* t;
  pqdts_ctx* ctx;
};

void on_stage(void* u, int32_t oiter, const double* X) {
  StageCtx* s = (StageCtx*)u;
  if (s->output >= 2) {
    const std::string name = pqdts::stage_file_name(0, oiter);
    printf(" %s\n", name.c_str());
    s->t->start("output");
    pqdts::write_state_file(name.c_str(), s->M, s->N, s->D, 0, X);
    s->t->stop("output");
  }
  const char* names[] = {"L", "dL", "BF", "CG", "Lalpha_min", "doproj", "doproj2", "conv_test"};
  for (const char* n : names) {
    double secs = 0;
    int64_t cnt = 0;
    if (pqdts_cuda_timer(s->ctx, n, &secs, &cnt) == PQDTS_OK && cnt > 0) s->t->set(n, secs, cnt);
  }
  s->t->print(oiter);
  fflush(stdout);
}

int fail(pqdts_ctx* c, const char* what) {
  char msg[1024] = {0};
  if (c) pqdts_cuda_last_error(c, msg, sizeof msg);
  fprintf(stderr, "pqdts_cuda.x: %s: %s\n", what, msg);
  return 1;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 15) {
    fprintf(stderr,
            "usage: %s M N D nnzF nnzP mode maxiter output gamma eps start_stage read_input smo_fact bench\n",
            argv[0]);
    return 1;
  }
  HostTimers t;
  t.start("prep");
  const int64_t M = atoll(argv[1]), N = atoll(argv[2]), D = atoll(argv[3]);
  const int64_t Fl = atoll(argv[4]), Pl = atoll(argv[5]);
  const int mode = atoi(argv[6]), maxiiter = atoi(argv[7]), output = atoi(argv[8]);
  const double gam = atof(argv[9]), conv_thres = atof(argv[10]);
  const int start_stage = atoi(argv[11]), read_input = atoi(argv[12]);
  const double smo_fact = atof(argv[13]);
  const int bench = atoi(argv[14]);
  const char* prec_env = getenv("PQDTS_PRECISION");
  const int precision = (prec_env && std::string(prec_env) == "mixed") ? PQDTS_MIXED : PQDTS_FP64;
  const char* dev_env = getenv("PQDTS_DEVICE");
  const int device = dev_env ? atoi(dev_env) : 0;

  ListLine().s("num_proc").i4(1).print();
  ListLine().s("M=").i8(M).s("N=").i8(N).s("D=").i8(D).print();
  ListLine().s("mode=").i4(mode).s("maxiiter=").i4(maxiiter).s("output=").i4(output).print();
  ListLine().s("gam=").r8(gam).s("smo_fact=").r8(smo_fact).print();
  ListLine().s("conv_thres=").r8(conv_thres).print();

  if (Fl < 0 && M != (D - 1) * (D - 1)) {
    ListLine().s("M is not (D-1)**2").print();
    return 0;
  }
  std::vector<int32_t> Fr, Fc, Pr, Pc;
  std::vector<double> Fv, Pv;
  if (Fl >= 0) {
    Fr.resize(Fl);
    Fc.resize(Fl);
    Fv.resize(Fl);
    if (!read_raw("data/F_row.bin", Fr.data(), Fl * 4) || !read_raw("data/F_col.bin", Fc.data(), Fl * 4) ||
        !read_raw("data/F_data.bin", Fv.data(), Fl * 8)) {
      fprintf(stderr, "pqdts_cuda.x: cannot read %lld entries from data/F_*.bin\n", (long long)Fl);
      return 1;
    }
    double s = 0;
    for (double v : Fv) s += v;
    ListLine().i4(0).s("sum(F)=").r8(s).print();
  }
  if (Pl >= 0) {
    Pr.resize(Pl);
    Pc.resize(Pl);
    Pv.resize(Pl);
    if (!read_raw("data/P_row.bin", Pr.data(), Pl * 4) || !read_raw("data/P_col.bin", Pc.data(), Pl * 4) ||
        !read_raw("data/P_data.bin", Pv.data(), Pl * 8)) {
      fprintf(stderr, "pqdts_cuda.x: cannot read %lld entries from data/P_*.bin\n", (long long)Pl);
      return 1;
    }
    double s = 0;
    for (double v : Pv) s += v;
    ListLine().i4(0).s("sum(P)=").r8(s).print();
  }

  pqdts_ctx* ctx = nullptr;
  if (pqdts_cuda_create(device, &ctx) != PQDTS_OK) return fail(ctx, "create");
  pqdts_cuda_set_verbose(ctx, 1);
  if (pqdts_cuda_set_problem_coo(ctx, M, N, D, Fl, Fr.data(), Fc.data(), Fv.data(), Pl, Pr.data(), Pc.data(),
                                 Pv.data(), gam, precision) != PQDTS_OK)
    return fail(ctx, "set_problem");
  Fr.clear(), Fc.clear(), Fv.clear(), Pr.clear(), Pc.clear(), Pv.clear();

  if (bench == 1) {
    // Operation timings (1581-1734) on the device, 10 repetitions each.
    ListLine().s("quick benchmark:").print();
    std::vector<double> tmp((size_t)M * N);
    const char* ops[] = {"L", "dL", "doproj", "Bdiag", "BF"};
    for (const char* op : ops)
      for (int r = 0; r < 10; ++r) {
        const double t1 = wall();
        double v = 0;
        int rc = PQDTS_OK;
        if (!strcmp(op, "L")) rc = pqdts_cuda_L(ctx, &v);
        else if (!strcmp(op, "dL")) rc = pqdts_cuda_dL(ctx, tmp.data()), v = tmp[0];
        else if (!strcmp(op, "doproj")) rc = pqdts_cuda_doproj(ctx);
        else if (!strcmp(op, "Bdiag")) rc = pqdts_cuda_Bdiag(ctx, tmp.data()), v = tmp[0];
        else rc = pqdts_cuda_BF(ctx, tmp.data(), tmp.data()), v = tmp[0];
        if (rc != PQDTS_OK) return fail(ctx, op);
        ListLine().s(std::string("t ") + op).r8(wall() - t1).r8(v).print();
      }
    std::vector<double> x0((size_t)M * N, 1.0 / (double)N);
    pqdts_cuda_set_x(ctx, x0.data());
  }

  // Restart (1840-1903).
  if (read_input == 1) {
    const char* path = "data/initial_     0.dat";
    FILE* f = fopen(path, "rb");
    if (f) {
      ListLine().s("reading starting state from").s(path).print();
      t.start("input");
      std::vector<char> rec;
      int64_t hdr[4];
      const char* what[4] = {"M", "N", "D", "localrows"};
      const int64_t want[4] = {M, N, D, M};
      for (int k = 0; k < 4; ++k) {
        if (!pqdts::read_record(f, rec) || rec.size() < 8) {
          fprintf(stderr, "pqdts_cuda.x: truncated header in %s\n", path);
          return 1;
        }
        memcpy(&hdr[k], rec.data(), 8);
        if (hdr[k] != want[k]) {
          ListLine().s("input file in this directory is for a different").s(what[k]).i8(want[k]).s("!=").i8(hdr[k]).print();
          return 0;
        }
      }
      int32_t rank2 = 0;
      if (!pqdts::read_record(f, rec) || rec.size() < 4) return 1;
      memcpy(&rank2, rec.data(), 4);
      if (rank2 != 0) {
        ListLine().s("input file in this directory is for a different rank").i4(0).s("!=").i4(rank2).print();
        return 0;
      }
      std::vector<double> X((size_t)M * N);
      if (!pqdts::read_record(f, rec) || rec.size() < X.size() * 8) {
        fprintf(stderr, "pqdts_cuda.x: %s holds fewer than M*N values\n", path);
        return 1;
      }
      memcpy(X.data(), rec.data(), X.size() * 8);
      fclose(f);
      t.stop("input");
      if (smo_fact > 0 && pqdts_cuda_smooth(M, N, smo_fact, X.data()) != PQDTS_OK) return fail(ctx, "smooth");
      if (pqdts_cuda_set_x(ctx, X.data()) != PQDTS_OK) return fail(ctx, "set_x");
    }
  }
  t.stop("prep");
  t.print(0);

  StageCtx sc{M, N, D, output, &t, ctx};
  double stats[PQDTS_NSTATS];
  t.start("min");
  if (pqdts_cuda_solve(ctx, mode, maxiiter, conv_thres, start_stage, output, on_stage, &sc, stats) != PQDTS_OK)
    return fail(ctx, "solve");
  t.stop("min");

  if (output >= 1) {
    const std::string name = pqdts::final_file_name(0);
    printf(" %s\n", name.c_str());
    std::vector<double> X((size_t)M * N);
    if (pqdts_cuda_get_x(ctx, X.data()) != PQDTS_OK) return fail(ctx, "get_x");
    t.start("output");
    if (!pqdts::write_state_file(name.c_str(), M, N, D, 0, X.data())) {
      fprintf(stderr, "pqdts_cuda.x: cannot write %s\n", name.c_str());
      return 1;
    }
    t.stop("output");
  }
  t.print(-1);
  pqdts_cuda_destroy(ctx);
  write_status();
  return 0;
}
