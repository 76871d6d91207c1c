// libpqdts_cuda.so: context, device memory, operations and the solver loop
// of the GB300 drop-in for pqdts's mode-1/mode-2 solve, behind the C ABI of
// include/pqdts_cuda.h.
//
// Control flow mirrors program pqdts (pqdts.f90:1908-2167) on the host; all
// vectors, scalars of the CG recurrence and every reduction stay on the
// device.  The host reads back only what decides a branch: the CG exit flag
// (polled once per queued chunk of iterations), the line-search objectives
// (one read per batch of step lengths), and the convergence value.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "../../include/pqdts_cuda.h"
#include "fortran_io.h"
#include "kernels.cuh"
#include "problem_host.h"
#include "tc_band.cuh"
#include "batch_cg.cuh"

namespace pqdts {

// Constants of the reference, float literals promoted as gfortran does.
const double kDx = (double)1e-5f;          // Lalpha_min*: dx (pqdts.f90:354, 404, 450)
const double kActiveTol = (double)1e-8f;   // tactivetol (1207)
const double kFeasTol = (double)1e-12f;    // xmin >= -1e-12 (424, 430)
const double kStage1Exit = (double)1e-4f;  // |dlalpha| < 1e-4 (1955)
const double kHuge = std::numeric_limits<double>::max();
constexpr int kMaxCG = 50;                 // do j = 1, 50 (2036)
constexpr int kMaxLS = 100;                // do i = 1, 100 (374, 420, 466)
constexpr int kBatchLS = 8;                // step lengths evaluated per sweep
constexpr int kElemGrid = 152 * 8;         // elementwise grids: 8 blocks per SM
constexpr size_t kCondatSmemMax = 200u * 1024u;  // Condat's rows staged in shared memory up to this size

struct Err : std::runtime_error {
  int code;
  Err(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(call)                                                                                        \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess)                                                                              \
      throw Err(e_ == cudaErrorMemoryAllocation ? PQDTS_E_NOMEM : PQDTS_E_CUDA,                         \
                std::string(#call) + ": " + cudaGetErrorString(e_) + " (" + __FILE__ + ":" +            \
                    std::to_string(__LINE__) + ")");                                                    \
  } while (0)

// Stream of the context whose entry point is running on this thread (set by
// the C-ABI wrapper): device arrays are allocated and freed stream-ordered on
// it (cudaMallocAsync / cudaFreeAsync), which, unlike cudaFree, does not
// synchronise the device -- contexts on other threads (the batched solve's
// workers) keep running.
static thread_local cudaStream_t t_alloc_stream = nullptr;

// Device array that keeps its allocation when a later problem fits in it
// (a context reused for a stream of instances allocates only when one grows).
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0, cap = 0;
  cudaStream_t s = nullptr;  // stream it was allocated on (null: cudaMalloc)
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) {
      if (s) cudaFreeAsync(p, s);
      else cudaFree(p);
    }
    p = nullptr;
    n = cap = 0;
    s = nullptr;
  }
  void alloc(size_t count) {
    if (count == 0) count = 1;
    if (p && count <= cap) {
      n = count;
      return;
    }
    release();
    s = t_alloc_stream;
    if (s) CK(cudaMallocAsync((void**)&p, count * sizeof(T), s));
    else CK(cudaMalloc((void**)&p, count * sizeof(T)));
    n = cap = count;
  }
  void upload(const T* h, size_t count, cudaStream_t s, std::atomic<int64_t>* bytes) {
    alloc(count);
    if (count) CK(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    if (bytes) *bytes += (int64_t)(count * sizeof(T));
  }
};

// GPU-time accumulators for the reference's timer names (pqdts.f90:103-186).
struct GpuTimers {
  struct Pending {
    int id;
    cudaEvent_t a, b;
  };
  std::vector<std::string> names;
  std::vector<double> secs;
  std::vector<int64_t> counts;
  std::vector<Pending> pending;
  std::vector<cudaEvent_t> pool;
  cudaStream_t st = nullptr;
  bool enabled = true;  // Scope regions recorded (off: no events at all)
  bool detail = false;  // also the per-kernel spans of a CG iteration ("CG.*")
  int id_of(const char* n) {
    for (size_t i = 0; i < names.size(); ++i)
      if (names[i] == n) return (int)i;
    names.push_back(n);
    secs.push_back(0);
    counts.push_back(0);
    return (int)names.size() - 1;
  }
  cudaEvent_t ev() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    return e;
  }
  // While a CUDA graph is being captured, spans become event-record nodes
  // of that graph (events owned by the graph, harvested after each replay).
  std::vector<Pending>* capture = nullptr;
  std::vector<cudaEvent_t> capture_pool;  // created before the capture began
  cudaEvent_t capture_ev() {
    cudaEvent_t e = nullptr;
    if (!capture_pool.empty()) {
      e = capture_pool.back();
      capture_pool.pop_back();
    } else if (cudaEventCreate(&e) != cudaSuccess) {
      e = nullptr;
    }
    return e;
  }
  int begin(const char* n) {
    if (capture) {
      Pending p{id_of(n), capture_ev(), nullptr};
      if (!p.a) throw Err(PQDTS_E_CUDA, "cudaEventCreate failed during graph capture");
      capture->push_back(p);
      CK(cudaEventRecordWithFlags(p.a, st, cudaEventRecordExternal));
      return -(int)capture->size();
    }
    Pending p{id_of(n), ev(), nullptr};
    CK(cudaEventRecord(p.a, st));
    pending.push_back(p);
    counts[p.id]++;
    return (int)pending.size() - 1;
  }
  // Spans of a graph replay that has completed (the stream was synchronised).
  void harvest(const std::vector<Pending>& spans) {
    for (const auto& p : spans) {
      float ms = 0;
      if (p.b) CK(cudaEventElapsedTime(&ms, p.a, p.b));
      secs[p.id] += ms * 1e-3;
      counts[p.id]++;
    }
  }
  // Called from destructors: never throws; a failed record only loses the
  // sample (the CUDA error itself surfaces at the next checked call).
  void end(int tok) noexcept {
    if (tok < 0) {
      if (!capture) return;
      Pending& p = (*capture)[-tok - 1];
      p.b = capture_ev();
      if (!p.b) return;
      if (cudaEventRecordWithFlags(p.b, st, cudaEventRecordExternal) != cudaSuccess) {
        cudaEventDestroy(p.b);
        p.b = nullptr;
      }
      return;
    }
    cudaEvent_t e = nullptr;
    if (!pool.empty()) {
      e = pool.back();
      pool.pop_back();
    } else if (cudaEventCreate(&e) != cudaSuccess) {
      return;
    }
    if (cudaEventRecord(e, st) != cudaSuccess) {
      pool.push_back(e);
      return;
    }
    pending[tok].b = e;
  }
  void flush() {
    if (pending.empty()) return;
    CK(cudaStreamSynchronize(st));
    for (auto& p : pending) {
      float ms = 0;
      if (p.b) {
        CK(cudaEventElapsedTime(&ms, p.a, p.b));
        pool.push_back(p.b);
      }
      secs[p.id] += ms * 1e-3;
      pool.push_back(p.a);
    }
    pending.clear();
  }
  ~GpuTimers() {
    for (auto& p : pending) {
      cudaEventDestroy(p.a);
      if (p.b) cudaEventDestroy(p.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
    for (auto e : capture_pool) cudaEventDestroy(e);
  }
};

struct Scope {
  static constexpr int kOff = INT_MIN;
  GpuTimers& t;
  int tok;
  Scope(GpuTimers& tt, const char* n) : t(tt), tok(tt.enabled ? tt.begin(n) : kOff) {}
  // a detail span: recorded only at timer level 2
  Scope(GpuTimers& tt, const char* n, bool detail)
      : t(tt), tok(tt.enabled && (!detail || tt.detail) ? tt.begin(n) : kOff) {}
  ~Scope() {
    if (tok != kOff) t.end(tok);
  }
};

// One captured chunk of CG iterations, replayed with a single graph launch;
// its kernel count and timer spans are credited per replay.
struct CGGraph {
  cudaGraphExec_t exec = nullptr;
  std::vector<GpuTimers::Pending> spans;
  int64_t kernels = 0;
  void destroy() noexcept {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    for (auto& p : spans) {
      if (p.a) cudaEventDestroy(p.a);
      if (p.b) cudaEventDestroy(p.b);
    }
    spans.clear();
  }
};

// Launch schedule of the banded products (autotuned per size bucket).
struct Schedule {
  int fwd_tile = 0;       // FP32 F.V tile: 0 = 64x64, 1 = 64x32, 2 = 32x32
  int trn_tile = 0;       // FP32 F^T.R tile (same codes) ...
  int trn_splits = 1;     // ... with its K range split in this many segments
  int trans_threads = 0;  // FP64 F^T product: threads per row block (0 = heuristic)
  int trans_cols = 0;     // ... and columns per thread
  int trans_rows = 0;     // 1: FP64 F^T product row-flattened (k_trans_rows)
  int fwd_rows = 0;       // 1: FP64 F.X product row-flattened (k_fwd_rows)
  int tuned = 0;          // 1 = picked by timing, 0 = heuristic
  int tc = 0;             // mixed CG products on the tensor cores (split-BF16x3)
  int tc_splits = 1;      // K segments of their F^T product
  int tc_bn = 0;          // their N tile width
  int tc_persistent = 0;  // 1: persistent warp-specialized kernel, 0: one CTA per tile
  int tc_splits1 = 1;     // K segments of their F.V product (> 1: FP32 partials + k_finish_t)
};

// Band operand of the tensor-core products: 128-row blocks of bf16 hi/lo
// values, block b covering K columns [kb[b], kb[b] + kTcK nch[b]), with the
// TMA maps of both halves (box kTcK x 128 rows, swizzled to the row width).
// Per-CTA tile lists of the persistent tensor-core kernel for one (N tile
// width, K splits) pair: CTA b takes tile[off[b] .. off[b+1]).
struct TcSched {
  DBuf<int32_t> off, tile;
  int grid = 0;
};

struct TcOperand {
  DBuf<__nv_bfloat16> hi, lo;
  DBuf<int32_t> kb, nch;
  std::vector<int32_t> h_nch;  // K chunks per row block (host copy: the tile costs)
  int blocks = 0, kmax = 0;
  CUtensorMap map_hi, map_lo;
  std::map<std::array<int, 3>, std::unique_ptr<TcSched>> scheds;  // keyed by (BN, splits, N)
};

// CG work vectors of one precision.
template <typename T>
struct CGBufs {
  DBuf<T> r, z, p, Hp, V, sn, rs, R2;
  void alloc(int64_t MN, int64_t M, int64_t DN) {
    r.alloc(MN);
    z.alloc(MN);
    p.alloc(MN);
    Hp.alloc(MN);
    V.alloc(MN);
    sn.alloc(MN);
    rs.alloc(M);
    R2.alloc(DN);
  }
};

}  // namespace pqdts

struct pqdts_ctx {
  int device = 0;
  cudaStream_t st = nullptr;
  std::string err;
  int verbose = 0;
  std::atomic<int64_t> launches{0};
  std::atomic<int64_t> h2d{0}, d2h{0};
  pqdts::HostProblem h;
  int precision = PQDTS_FP64;
  bool have_problem = false;
  // problem on the device
  pqdts::DBuf<int32_t> flo, fw, tidx;
  pqdts::DBuf<int64_t> foff, tptr;
  pqdts::DBuf<double> fval, tval, bdiag, P;
  pqdts::DBuf<float> fval32, tval32, tbval32, rsq32;
  pqdts::DBuf<double> sqd;  // sqrt(bdfac * Bdiag) per row, FP64 CG step
  bool t_contiguous = false;  // every column of F supported on a contiguous range of d
  pqdts::DBuf<unsigned> counters;  // grid-completion counters of fused reductions (kept at 0 between launches)
  pqdts::DBuf<int32_t> tlo, tw;
  pqdts::DBuf<int64_t> toff;
  // iterate and work arrays
  pqdts::DBuf<double> X, G, Xc, R, sn64;
  pqdts::DBuf<int8_t> ik;
  pqdts::DBuf<int32_t> maxr;
  pqdts::CGBufs<double> cg64;
  pqdts::CGBufs<float> cg32;
  pqdts::DBuf<double> part, part2, sc, alphas, lsout, cglog;
  // reference-order reductions (FP64 path): residual stack, Condat scratch,
  // per-row / per-column chain results
  pqdts::DBuf<double> Rst, aux, srow, gcol, colbuf, lred;
  // mixed-precision line search: alpha = 0 candidate, its residual (FP32),
  // candidate differences and their banded products (FP32)
  pqdts::DBuf<double> x0c;
  pqdts::DBuf<float> r0_32, d32, fdx32, hpart32;
  pqdts::DBuf<double> Gf;  // mixed path: full-space gradient of X (version Gf_ver)
  int64_t Gf_ver = -1;
  // mixed path: double-FP32 banded products for the gradient and the FP64
  // objective checks (option -1 auto = on, 0 native FP64, 1 on): F and F^T
  // values, and the split X and R operands, as (hi, lo) pairs
  pqdts::DBuf<float2> fdf, tdf, xdf, rdf;
  // row-occupancy masks of the double-FP32 forward products' operand
  // (k_row_masks, up to kBatchLS stacked inputs)
  pqdts::DBuf<uint32_t> xmask;
  // Zero-skipping products (option row_masks, on unless 0; only where F is
  // finite).  The transposed FP64 products: F^T in tiles of 32 rows
  // (k_ftile_build; built when every column of F is contiguous in d) and R's
  // column masks and occupied-row lists (k_col_index)
  pqdts::DBuf<uint32_t> rmask;
  pqdts::DBuf<double> ftile;
  pqdts::DBuf<int32_t> ftile_lo, ftile_hi, ccnt, clist;
  pqdts::DBuf<int64_t> ftile_off;
  // the forward FP64 products with masks: F in tiles of 32 rows
  // (k_fwtile_build; built when F is finite) and X's column masks and
  // occupied-row lists for up to kBatchLS stacked inputs
  pqdts::DBuf<double> fwtile;
  pqdts::DBuf<int32_t> fwtile_lo, fwtile_hi, xccnt, xclist;
  pqdts::DBuf<int64_t> fwtile_off;
  pqdts::DBuf<uint32_t> xcmask;
  int mask_option = 1;
  // option count_fmas: the masked FP64 products add the FMAs they execute
  // (per output lane) to fmacount[0] (forward) and [1] (transposed)
  bool count_fmas = false;
  pqdts::DBuf<unsigned long long> fmacount;
  bool f_finite = true;
  int df_option = -1;
  int df_rows = 0;  // band rows per block of the double-FP32 products (0: chosen by size)
  bool df_fwd = false, df_trans = false;
  bool exact = true;  // FP64: every reduction in the oracle's order
  pqdts::DBuf<int> ipart;
  pqdts::DBuf<long long> icount;
  double* pin = nullptr;  // pinned host scalars
  bool fullspace = true;
  std::vector<int32_t> h_maxr;
  pqdts::GpuTimers timers;
  int64_t n_cg = 0, n_lsL = 0, n_refine = 0;
  bool refine = false;  // mixed precision: FP64 CG from now on
  int refine_option = 0;  // 1: mixed precision runs the FP64 CG for all of stage 2
  int internal_f_option = -1;  // internal F on the device: -1 for mixed problems, 0 never (host), 1 always
  double target_L = 0.0;  // optional objective stopping rule (0 = off)
  // version of X, bumped on every write; results keyed on it are reused
  int64_t xver = 0, R_ver = -1, G_ver = -1, L_ver = -1, rebuilt_ver = -1;
  bool G_full = true;
  double L_cache = 0.0, Lgam_cache = 0.0;  // L of X (version L_ver) and its gamma term
  bool target_hit = false;
  // last batch of FP64-evaluated line-search candidates (Xc, Rst = O - P):
  // step lengths, objectives (+ gamma part), xmin, for X of version cand_xver
  int64_t cand_xver = -1;
  int cand_B = 0;
  bool cand_stage2 = false;
  double cand_alpha[8], cand_L[8], cand_Lgam[8], cand_xmin[8];
  // CG chunks captured as CUDA graphs (keyed by variant; dropped whenever the
  // device buffers are reallocated) and the products' launch schedule
  std::map<std::array<uint64_t, 5>, pqdts::CGGraph> graphs;
  bool use_graphs = true;
  bool autotune = true;
  // tensor-core Hessian products of the mixed CG: option (-1 auto, 0 off,
  // 1 on), operands F and F^T, the split B operands V^T and (2 F.V)^T
  int tc_option = -1;
  int tc_persistent_option = -1;  // -1 autotuned, 0 one CTA per tile, 1 persistent
  int tc_splits1_option = -1;     // -1 autotuned, else the K segments of the tensor-core F.V product
  uint64_t tc_wait_ns = pqdts::kTcWaitNs;  // limit of each mbarrier wait in the tensor-core kernels
  int tc_wait_probe = 0;                   // 1: their producer waits on a barrier nothing arrives on (test hook)
  int rows_option = -1;           // row-flattened FP64 products: -1 autotuned, 0 never, 1 always (where they apply)
  int num_sms = 0;
  bool tc_ready = false;
  int tc_bn = 0, tc_stages = 0;
  int64_t tc_mp = 0, tc_dp = 0;  // row strides (elements) of V^T and (F.V)^T
  pqdts::TcOperand tcF, tcFt;
  pqdts::DBuf<__nv_bfloat16> vt_hi, vt_lo, yt_hi, yt_lo;
  pqdts::DBuf<float> ypart;  // FP32 partials of F.V when its K range is split
  CUtensorMap map_vt_hi, map_vt_lo, map_yt_hi, map_yt_lo;
  // the line search's probes dX^T split (kBatchLS * N rows of tc_mp) for
  // their F products on the tensor cores, and its maps (built for the tile
  // width, buffer and stride recorded beside them)
  pqdts::DBuf<__nv_bfloat16> ls_hi, ls_lo;
  CUtensorMap map_ls_hi, map_ls_lo;
  int ls_map_bn = 0;
  const void* ls_map_ptr = nullptr;
  int64_t ls_map_mp = 0, ls_map_rows = 0;
  int tc_screen_option = -1;  // line-search screen on the tensor cores: -1 auto (with the CG's), 0 off
  pqdts::Schedule sched;
  bool own_stream = true;  // false: a member of a batched group, on the group's stream
  // group context of a batched lockstep solve: the members' CG table
  pqdts::DBuf<pqdts::CGMember> memtab;
  std::vector<pqdts::CGMember> h_memtab;
  void drop_graphs() noexcept {
    for (auto& kv : graphs) kv.second.destroy();
    graphs.clear();
  }
  ~pqdts_ctx() { drop_graphs(); }
};

namespace pqdts {

using Ctx = pqdts_ctx;

// Scratch of pqdts_cuda_simplexproj_noalloc: Condat's per-row working lists.
// In host code this name is only a stand-in for the symbol; the device
// address comes from cudaGetSymbolAddress, once per device and CUDA context
// (the context's unique id is kept with it: a device reset or a caller's own
// driver-API context on the same device gets its own lookup).
static __device__ __align__(256) double g_noalloc_scratch[PQDTS_NOALLOC_SCRATCH];
constexpr int kMaxDevices = 64;
static std::mutex g_noalloc_mu;
struct NoallocSlot {
  double* ptr = nullptr;
  unsigned long long ctx_id = 0;
};
static NoallocSlot g_noalloc[kMaxDevices];

// Unique id of the calling thread's current CUDA context (0: none or the
// driver entry points are unavailable -- then the address is looked up on
// every call, which allocates nothing either).
static unsigned long long current_ctx_id() {
  typedef CUresult (*GetCurrentFn)(CUcontext*);
  typedef CUresult (*GetIdFn)(CUcontext, unsigned long long*);
  static std::once_flag once;
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = (GetCurrentFn)p;
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = (GetIdFn)p;
  });
  if (!get_current || !get_id) return 0;
  CUcontext cur = nullptr;
  unsigned long long id = 0;
  if (get_current(&cur) != CUDA_SUCCESS || cur == nullptr || get_id(cur, &id) != CUDA_SUCCESS) return 0;
  return id;
}

static DevBands bands_of(Ctx& c) {
  DevBands b;
  b.M = (int)c.h.M;
  b.N = (int)c.h.N;
  b.D = (int)c.h.D;
  b.flo = c.flo.p;
  b.fw = c.fw.p;
  b.foff = c.foff.p;
  b.tptr = c.tptr.p;
  b.tidx = c.tidx.p;
  return b;
}

static inline int cdiv(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// X changed: results keyed on the old version are stale.
static void touch_x(Ctx& c) { c.xver++; }

static void post_launch(Ctx& c) {
  c.launches++;
  CK(cudaGetLastError());
}

static int elem_grid(int64_t total) { return std::max(1, std::min<int>(kElemGrid, cdiv(total, 256))); }

static void reduce_to(Ctx& c, const double* part, int64_t count, double* out, int B = 1, bool is_min = false,
                      double init = 0.0, const double* pred = nullptr) {
  if (is_min) k_reduce<true><<<B, 512, 0, c.st>>>(part, count, out, init, pred);
  else k_reduce<false><<<B, 512, 0, c.st>>>(part, count, out, init, pred);
  post_launch(c);
}

static void read_back(Ctx& c, const double* dev, int count) {
  CK(cudaMemcpyAsync(c.pin, dev, count * sizeof(double), cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
}

// After a read-back of the scalars: a tensor-core kernel whose bounded
// barrier wait ran out has set SC_TCERR.  The flag is cleared (the kernels
// freed their tensor memory and stored nothing, the context stays usable)
// and the call fails with PQDTS_E_CUDA.
static void check_tc_error(Ctx& c) {
  if (c.pin[SC_TCERR] == 0.0) return;
  CK(cudaMemsetAsync(c.sc.p + SC_TCERR, 0, sizeof(double), c.st));
  CK(cudaStreamSynchronize(c.st));
  throw Err(PQDTS_E_CUDA, "tensor-core product: a barrier wait timed out");
}

// ---------------------------------------------------------------------------
// Problem upload and buffer allocation.
// ---------------------------------------------------------------------------
// Band rows per block of the double-FP32 products: the most of 8, 4, 2
// that still gives >= 40 warps per SM to cover the operand loads' latency
// (measured: M=2000, N=200, D=4000 runs best at 4 rows for F.X and 2 for
// F^T.R; M=10^4, N=10^3, D=2*10^4 at 8); rbopt > 0: that, as 2/4/8.
static int df_rows_per_block(int64_t rows, int N, int rbopt, int sms) {
  if (rbopt > 0) return rbopt >= 8 ? 8 : (rbopt >= 4 ? 4 : 2);
  const int64_t wpr = cdiv(N, 32);
  for (int rb : {8, 4})
    if ((rows + rb - 1) / rb * wpr >= (int64_t)40 * sms) return rb;
  return 2;
}

template <int MODE>
static void launch_fwd_df(Ctx& c, double* R, const uint32_t* xmask) {
  const int N = (int)c.h.N, D = (int)c.h.D;
  const int rb = df_rows_per_block(D, N, c.df_rows, c.num_sms);
  const int threads = 32 * std::min(kDfColWarps, cdiv(N, 32));
  const dim3 grid(cdiv(D, rb), cdiv(N, threads));
  DevBands bd = bands_of(c);
  if (rb == 8) k_fwd_df<MODE, 8><<<grid, threads, 0, c.st>>>(bd, c.fdf.p, c.xdf.p, c.P.p, R, xmask);
  else if (rb == 4) k_fwd_df<MODE, 4><<<grid, threads, 0, c.st>>>(bd, c.fdf.p, c.xdf.p, c.P.p, R, xmask);
  else k_fwd_df<MODE, 2><<<grid, threads, 0, c.st>>>(bd, c.fdf.p, c.xdf.p, c.P.p, R, xmask);
  post_launch(c);
}


// (hi, lo) FP32 pair of an FP64 value, as k_split_df forms it on the device.
static float2 split_df_host(double v) {
  const float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}

static void setup_device(Ctx& c) {
  HostProblem& h = c.h;
  const int64_t M = h.M, N = h.N, D = h.D, MN = M * N;
  c.drop_graphs();  // their kernels hold the buffers about to be replaced
  c.flo.upload(h.flo.data(), D, c.st, &c.h2d);
  c.fw.upload(h.fw.data(), D, c.st, &c.h2d);
  c.foff.upload(h.foff.data(), D, c.st, &c.h2d);
  c.fval.upload(h.fval.data(), h.fval.size(), c.st, &c.h2d);
  c.tptr.upload(h.tptr.data(), h.tptr.size(), c.st, &c.h2d);
  c.tidx.upload(h.tidx.data(), h.tidx.size(), c.st, &c.h2d);
  c.tval.upload(h.tval.data(), h.tval.size(), c.st, &c.h2d);
  c.bdiag.upload(h.bdiag.data(), M, c.st, &c.h2d);
  c.P.upload(h.P.data(), h.P.size(), c.st, &c.h2d);
  c.t_contiguous = true;
  for (int64_t i = 0; i < M && c.t_contiguous; ++i) {
    const int64_t e0 = h.tptr[i], e1 = h.tptr[i + 1];
    if (e1 > e0 && h.tidx[e1 - 1] - h.tidx[e0] + 1 != e1 - e0) c.t_contiguous = false;
  }
  if (c.precision == PQDTS_MIXED) {
    std::vector<float> f32(h.fval.begin(), h.fval.end());
    c.fval32.upload(f32.data(), f32.size(), c.st, &c.h2d);
    std::vector<float> t32(h.tval.begin(), h.tval.end());
    c.tval32.upload(t32.data(), t32.size(), c.st, &c.h2d);
    transposed_bands(h);
    c.tlo.upload(h.tlo.data(), h.tlo.size(), c.st, &c.h2d);
    c.tw.upload(h.tw.data(), h.tw.size(), c.st, &c.h2d);
    c.toff.upload(h.toff.data(), h.toff.size(), c.st, &c.h2d);
    std::vector<float> tb32(h.tbval.begin(), h.tbval.end());
    c.tbval32.upload(tb32.data(), tb32.size(), c.st, &c.h2d);
    c.rsq32.alloc(M);
    c.cg32.alloc(MN, M, D * N);
    c.x0c.alloc(MN);
    c.Gf.alloc(MN);
    c.r0_32.alloc(D * N);
    c.d32.alloc((size_t)kBatchLS * MN);
    c.fdx32.alloc((size_t)kBatchLS * D * N);
    c.df_fwd = c.df_option != 0;
    c.df_trans = c.df_fwd && c.t_contiguous;
    CK(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, c.device));
    if (c.df_fwd) {
      std::vector<float2> fd(h.fval.size());
      for (size_t k = 0; k < fd.size(); ++k) fd[k] = split_df_host(h.fval[k]);
      c.fdf.upload(fd.data(), fd.size(), c.st, &c.h2d);
      c.xdf.alloc(MN);
    } else {
      c.fdf.release();
      c.xdf.release();
    }
    if (c.df_trans) {
      std::vector<float2> td(h.tval.size());
      for (size_t k = 0; k < td.size(); ++k) td[k] = split_df_host(h.tval[k]);
      c.tdf.upload(td.data(), td.size(), c.st, &c.h2d);
      c.rdf.alloc(D * N);
    } else {
      c.tdf.release();
      c.rdf.release();
    }
    CK(cudaStreamSynchronize(c.st));  // host staging vectors go out of scope
  } else {
    c.fval32.release();
    c.tval32.release();
    c.tbval32.release();
    c.fdf.release();
    c.tdf.release();
    c.xdf.release();
    c.rdf.release();
    c.df_fwd = c.df_trans = false;
  }
  c.cg64.alloc(MN, M, D * N);
  c.sqd.alloc(M);
  c.f_finite = std::all_of(h.fval.begin(), h.fval.end(), [](double v) { return std::isfinite(v); });
  c.xmask.alloc((size_t)kBatchLS * cdiv(N, 32) * cdiv(M, 32));
  c.rmask.alloc((size_t)N * cdiv(D, 32));
  if (c.t_contiguous && c.f_finite) {
    // F^T's 32-row tiles: the union of the tile's column ranges of d each
    const int64_t nb = cdiv(M, 32);
    std::vector<int32_t> lo(nb), hi(nb);
    std::vector<int64_t> off(nb + 1, 0);
    for (int64_t b = 0; b < nb; ++b) {
      int32_t l = INT32_MAX, u = 0;
      for (int64_t i = b * 32; i < std::min(M, b * 32 + 32); ++i) {
        const int64_t e0 = h.tptr[i], e1 = h.tptr[i + 1];
        if (e1 > e0) {
          l = std::min(l, h.tidx[e0]);
          u = std::max(u, h.tidx[e1 - 1] + 1);
        }
      }
      if (l >= u) l = u = 0;
      lo[b] = l;
      hi[b] = u;
      off[b + 1] = off[b] + (int64_t)(u - l) * 32;
    }
    c.ftile_lo.upload(lo.data(), nb, c.st, &c.h2d);
    c.ftile_hi.upload(hi.data(), nb, c.st, &c.h2d);
    c.ftile_off.upload(off.data(), nb + 1, c.st, &c.h2d);
    c.ftile.alloc(std::max<int64_t>(off[nb], 1));
    k_ftile_build<<<(unsigned)nb, 256, 0, c.st>>>(bands_of(c), c.tval.p, c.ftile_lo.p, c.ftile_hi.p, c.ftile_off.p,
                                                   c.ftile.p);
    post_launch(c);
    c.ccnt.alloc((size_t)N * (cdiv(D, 32) + 1));
    c.clist.alloc((size_t)N * D);
  } else {
    c.ftile.release();
    c.ftile_lo.release();
    c.ftile_hi.release();
    c.ftile_off.release();
    c.ccnt.release();
    c.clist.release();
  }
  if (c.f_finite) {
    // F's 32-row tiles: the union of the tile's row bands each
    const int64_t nb = cdiv(D, 32);
    std::vector<int32_t> lo(nb), hi(nb);
    std::vector<int64_t> off(nb + 1, 0);
    for (int64_t b = 0; b < nb; ++b) {
      int32_t l = INT32_MAX, u = 0;
      for (int64_t d = b * 32; d < std::min(D, b * 32 + 32); ++d) {
        if (h.flo[d] >= 0 && h.fw[d] > 0) {
          l = std::min(l, h.flo[d]);
          u = std::max(u, h.flo[d] + h.fw[d]);
        }
      }
      if (l >= u) l = u = 0;
      lo[b] = l;
      hi[b] = u;
      off[b + 1] = off[b] + (int64_t)(u - l) * 32;
    }
    c.fwtile_lo.upload(lo.data(), nb, c.st, &c.h2d);
    c.fwtile_hi.upload(hi.data(), nb, c.st, &c.h2d);
    c.fwtile_off.upload(off.data(), nb + 1, c.st, &c.h2d);
    c.fwtile.alloc(std::max<int64_t>(off[nb], 1));
    k_fwtile_build<<<(unsigned)nb, 256, 0, c.st>>>(bands_of(c), c.fval.p, c.fwtile_lo.p, c.fwtile_hi.p,
                                                    c.fwtile_off.p, c.fwtile.p);
    post_launch(c);
    c.xcmask.alloc((size_t)kBatchLS * N * cdiv(M, 32));
    c.xccnt.alloc((size_t)kBatchLS * N * (cdiv(M, 32) + 1));
    c.xclist.alloc((size_t)kBatchLS * N * M);
    CK(cudaStreamSynchronize(c.st));  // host staging vectors go out of scope
  } else {
    c.fwtile.release();
    c.fwtile_lo.release();
    c.fwtile_hi.release();
    c.fwtile_off.release();
    c.xcmask.release();
    c.xccnt.release();
    c.xclist.release();
  }
  c.fmacount.alloc(2);
  CK(cudaMemsetAsync(c.fmacount.p, 0, 2 * sizeof(unsigned long long), c.st));
  CK(cudaFuncSetAttribute(k_condat_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCondatSmemMax));
  CK(cudaFuncSetAttribute(k_simplex_smem, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCondatSmemMax));
  c.counters.alloc(8);
  CK(cudaMemsetAsync(c.counters.p, 0, 8 * sizeof(unsigned), c.st));
  c.exact = (c.precision == PQDTS_FP64);
  // residual stack of the line-search candidates (both precisions)
  c.Rst.alloc((size_t)kBatchLS * D * N);
  // Condat scratch rows (FP64 path only; the mixed path projects in place)
  if (c.exact) c.aux.alloc((size_t)kBatchLS * MN);
  else c.aux.release();
  c.srow.alloc((size_t)kBatchLS * std::max(D, M));
  c.gcol.alloc((size_t)kBatchLS * N);
  c.colbuf.alloc(2 * N);
  c.lred.alloc(kBatchLS);
  c.X.alloc(MN);
  c.G.alloc(MN);
  c.Xc.alloc((size_t)kBatchLS * MN);
  c.R.alloc(D * N);
  c.sn64.alloc(MN);
  c.ik.alloc(MN);
  c.maxr.alloc(M);
  const int64_t fwd_parts = (int64_t)cdiv(N, kBX) * cdiv(D, kBY) * kBatchLS;
  const int64_t np = std::max<int64_t>({fwd_parts, M, (int64_t)kElemGrid * kBatchLS, 1024});
  c.part.alloc(np);
  c.part2.alloc(np);
  c.ipart.alloc(kElemGrid);
  c.icount.alloc(1);
  c.sc.alloc(SC_NSC);
  CK(cudaMemsetAsync(c.sc.p, 0, SC_NSC * sizeof(double), c.st));
  c.alphas.alloc(kBatchLS);
  c.lsout.alloc(4 * kBatchLS);
  c.cglog.alloc(4 * kMaxCG);
  // Initial X = 1/N (pqdts.f90:1834-1838) and maxr from the seeded stream.
  k_fill<<<elem_grid(MN), 256, 0, c.st>>>(MN, 1.0 / (double)N, c.X.p);
  post_launch(c);
  c.R_ver = c.G_ver = c.L_ver = c.rebuilt_ver = c.Gf_ver = -1;
  touch_x(c);
  CK(cudaMemcpyAsync(c.maxr.p, c.h_maxr.data(), M * 4, cudaMemcpyHostToDevice, c.st));
  c.h2d += M * 4;
  CK(cudaStreamSynchronize(c.st));
  c.fullspace = true;
  c.have_problem = true;
}

static void need_problem(Ctx& c) {
  if (!c.have_problem) throw Err(PQDTS_E_STATE, "no problem set (call pqdts_cuda_set_problem first)");
}

// ---------------------------------------------------------------------------
// Operations on device arrays.
// ---------------------------------------------------------------------------
static void rebuild(Ctx& c, double* X, int B = 1) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  k_rebuild_t<<<dim3(cdiv(M, 32), B), kTileThreads, 0, c.st>>>(X, (int64_t)M * N, c.maxr.p, M, N);
  post_launch(c);
}

// Objective from the per-row residual sums srow[b][d] of B matrices Xs
// (L_red) plus the gamma term of Xs (L_gam, 954-964) -> lsout[b].  FP64 path:
// rows added in ascending order, then the gamma term's column chains added
// column by column (the oracle's order).  Mixed path: fixed-shape trees.
static void objective_combine(Ctx& c, const double* Xs, int B) {
  const int M = (int)c.h.M, N = (int)c.h.N, D = (int)c.h.D;
  if (c.exact) {
    double* out = c.h.gam != 0 ? c.lred.p : c.lsout.p;
    k_seqsum<<<B, 32, 0, c.st>>>(c.srow.p, D, nullptr, out, B, nullptr);
    post_launch(c);
    if (c.h.gam != 0) {
      k_colchain<1><<<dim3(cdiv(N, kChainWarps), B), 32 * kChainWarps, 0, c.st>>>(
          Xs, nullptr, (int64_t)M * N, M, N, c.h.gam, c.gcol.p, nullptr, nullptr);
      post_launch(c);
      k_seqsum<<<B, 32, 0, c.st>>>(c.gcol.p, N, c.lred.p, c.lsout.p, B, nullptr);
      post_launch(c);
    }
    CK(cudaMemsetAsync(c.lsout.p + kBatchLS, 0, B * sizeof(double), c.st));
    return;
  }
  reduce_to(c, c.srow.p, D, c.lsout.p, B);
  if (c.h.gam != 0) {
    const int g = elem_grid((int64_t)(M - 1) * N);
    k_gamma_part<<<dim3(g, B), 256, 0, c.st>>>(Xs, (int64_t)M * N, M, N, c.h.gam, c.part2.p);
    post_launch(c);
    reduce_to(c, c.part2.p, g, c.lsout.p + kBatchLS, B);
  } else {
    CK(cudaMemsetAsync(c.lsout.p + kBatchLS, 0, B * sizeof(double), c.st));
  }
}

// Objective of B stacked, already projected/rebuilt candidates: O - P of
// each into the residual stack, per-row chains, then objective_combine.
static void require(const void* p, const char* what) {
  if (p == nullptr) throw Err(PQDTS_E_STATE, std::string("internal: device buffer ") + what + " is not allocated");
}

// Rows per block of the row-flattened products: the most busy lanes with
// RB*N <= 1024 threads and RB <= 32; 0 when N is outside [32, 1024].
static int rows_per_block(int N) {
  if (N < 32 || N > 1024) return 0;
  int best = 0;
  double beff = 0.0;
  for (int rb = 1; rb <= 32 && rb * N <= 1024; ++rb) {
    const int t = rb * N;
    const double eff = (double)t / (32.0 * ((t + 31) / 32));
    if (eff > beff + 1e-12) {
      beff = eff;
      best = rb;
    }
  }
  return best;
}

// F.X (B stacked inputs, xstride apart) with the epilogue MODE of k_fwd, in
// the context's form: column-tiled, or row-flattened (rows = 1; the same bits).
template <typename T, int MODE>
static void launch_fwd(Ctx& c, const T* fv, const T* X, int64_t xstride, const double* P, T* R, int B,
                       const double* pred, int rows = -1) {
  const int N = (int)c.h.N, D = (int)c.h.D;
  DevBands bd = bands_of(c);
  const int RB = rows_per_block(N);
  if constexpr (std::is_same<T, double>::value) {
    if (c.mask_option != 0 && c.fwtile.p != nullptr && fv == c.fval.p) {
      // FP64: (column n, 32-row tile of F) warps visiting only the rows of
      // X where X[i, n] != 0 (X's column lists; the same bits)
      const int M = (int)c.h.M;
      k_col_index<T><<<dim3(cdiv(N, kIndexWarps), B), 32 * kIndexWarps, 0, c.st>>>(X, xstride, M, N, c.xcmask.p,
                                                                                  c.xccnt.p, c.xclist.p);
      post_launch(c);
      k_fwd_col<T, MODE><<<dim3(cdiv(N, kTcWarps), cdiv(D, 32), B), dim3(32, kTcWarps), 0, c.st>>>(
          M, N, D, c.fwtile.p, c.fwtile_lo.p, c.fwtile_hi.p, c.fwtile_off.p, X, xstride, c.xcmask.p, c.xccnt.p,
          c.xclist.p, P, R, pred, c.count_fmas ? c.fmacount.p : nullptr);
      post_launch(c);
      return;
    }
  }
  if ((rows < 0 ? c.sched.fwd_rows : rows) && RB > 0) {
    const int threads = cdiv((int64_t)RB * N, 32) * 32;
    k_fwd_rows<T, MODE><<<dim3(cdiv(D, RB), B), threads, 0, c.st>>>(bd, fv, X, xstride, P, R, RB, pred);
  } else {
    k_fwd<T, MODE><<<dim3(cdiv(N, kBX), cdiv(D, kBY), B), dim3(kBX, kBY), 0, c.st>>>(bd, fv, X, xstride, P, R, nullptr,
                                                                                    pred);
  }
  post_launch(c);
}


// Residual of X (FP64, M x N) in double-FP32: MODE 0 R = 2*(F.X - P),
// MODE 3 R = F.X - P.
template <int MODE>
static void fwd_df(Ctx& c, const double* X, double* R) {
  const int64_t MN = c.h.M * c.h.N;
  require(c.xdf.p, "xdf");
  k_split_df<<<elem_grid(MN), 256, 0, c.st>>>(X, MN, 1.0, c.xdf.p);
  post_launch(c);
  const uint32_t* xm = nullptr;
  if (c.mask_option != 0 && c.f_finite) {
    // X's row-occupancy masks: the product visits only rows where a warp's
    // columns are non-zero
    const int M = (int)c.h.M, ng = cdiv(c.h.N, 32), nseg = cdiv(M, 32);
    k_row_masks<double><<<dim3(cdiv((int64_t)ng * nseg * 32, 256), 1), 256, 0, c.st>>>(X, 0, M, (int)c.h.N, c.xmask.p);
    post_launch(c);
    xm = c.xmask.p;
  }
  launch_fwd_df<MODE>(c, R, xm);
}

static void objective_stack(Ctx& c, const double* Xs, int B) {
  const int M = (int)c.h.M, N = (int)c.h.N, D = (int)c.h.D;
  require(c.Rst.p, "Rst");
  if (B < 1 || B > kBatchLS) throw Err(PQDTS_E_STATE, "internal: candidate batch out of range");
  if (c.df_fwd) {
    for (int b = 0; b < B; ++b) fwd_df<3>(c, Xs + (size_t)b * M * N, c.Rst.p + (size_t)b * D * N);
  } else {
    launch_fwd<double, 3>(c, c.fval.p, Xs, (int64_t)M * N, c.P.p, c.Rst.p, B, nullptr);
  }
  k_rowchain_resid_t<<<dim3(cdiv(D, 32), B), kTileThreads, 0, c.st>>>(c.Rst.p, c.flo.p, D, N, 1.0, c.srow.p);
  post_launch(c);
  objective_combine(c, Xs, B);
}

static void fetch_objectives(Ctx& c, int B, double* L) {
  CK(cudaMemcpyAsync(c.pin, c.lsout.p, 4 * kBatchLS * sizeof(double), cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  for (int b = 0; b < B; ++b) L[b] = (c.h.gam != 0 && !c.exact) ? c.pin[b] + c.pin[kBatchLS + b] : c.pin[b];
}

// Max-column rebuild of the context's X.  FP64 path: always a new version
// of X (across M rows some row practically always moves by an ulp, and the
// trajectory must stay bit-exact).  Mixed path: re-applying the rebuild to
// an X that is already consistent with maxr only moves values by ulps, so
// results computed for that X stay in use.
static void rebuild_x(Ctx& c) {
  rebuild(c, c.X.p);
  if (!c.exact && c.rebuilt_ver == c.xver) return;
  touch_x(c);
  c.rebuilt_ver = c.xver;
}

// R = 2*(O - P) with O = F.X for the context's X, unless R already holds it
// for this version of X.
static void ensure_R(Ctx& c) {
  if (c.R_ver == c.xver) return;
  if (c.df_fwd) fwd_df<0>(c, c.X.p, c.R.p);
  else launch_fwd<double, 0>(c, c.fval.p, c.X.p, 0, c.P.p, c.R.p, 1, nullptr);
  c.R_ver = c.xver;
}

// L(X) on the context's X (917-973).  The residual sums come from R (exactly
// O - P = R/2), so L and dL of one X share one banded product.
static double op_L(Ctx& c) {
  Scope s(c.timers, "L");
  if (!c.fullspace) rebuild_x(c);
  if (c.L_ver == c.xver) return c.L_cache;
  ensure_R(c);
  const int D = (int)c.h.D, N = (int)c.h.N;
  k_rowchain_resid_t<<<dim3(cdiv(D, 32), 1), kTileThreads, 0, c.st>>>(c.R.p, c.flo.p, D, N, 0.5, c.srow.p);
  post_launch(c);
  objective_combine(c, c.X.p, 1);
  double L;
  fetch_objectives(c, 1, &L);
  c.L_cache = L;
  c.Lgam_cache = (c.h.gam != 0 && !c.exact) ? c.pin[kBatchLS] : 0.0;
  c.L_ver = c.xver;
  return L;
}

// Block shape of k_trans: threads x C columns per pass with the fewest idle
// lanes (an idle lane still costs its FP64 issue slot).
struct TransShape {
  int threads, C;
  int rows = 0;  // 1: the row-flattened kernel (k_trans_rows)
};


static TransShape trans_shape(int N) {
  // fewest passes over the CSR row first (each pass re-reads it), then the
  // fewest idle lanes, then the fewest columns per thread (more warps).
  TransShape best{32, 1};
  int64_t best_passes = INT64_MAX, best_waste = INT64_MAX;
  for (int C : {1, 2, 4, 8})
    for (int t = 32; t <= 256; t += 32) {
      const int64_t per = (int64_t)t * C;
      const int64_t passes = (N + per - 1) / per;
      const int64_t waste = passes * per - N;
      if (passes < best_passes || (passes == best_passes && waste < best_waste)) {
        best_passes = passes;
        best_waste = waste;
        best = {t, C};
      }
    }
  return best;
}

// k_trans with an explicit block shape (every shape gives the same values:
// each output accumulates its CSR row in ascending order in one thread).
template <typename T, bool HVP>
static void launch_trans_shape(Ctx& c, TransShape sh, const T* tv, const T* R, const T* V, const T* rs, int reduced,
                               T c2gam, const int8_t* ik, T* G, const T* W, double* dpart, const double* pred,
                               T* Gf = nullptr) {
  const int M = (int)c.h.M;
  DevBands bd = bands_of(c);
  const int RB = rows_per_block((int)c.h.N);
  int raw = 0;
  if constexpr (std::is_same<T, double>::value) {
    if (c.mask_option != 0 && c.ftile.p != nullptr && tv == c.tval.p) {
      // FP64: the sums by (column n, 32-row tile of F^T) warps visiting only
      // the d where R[d, n] != 0 (R's column lists; the same bits), then
      // k_trans's epilogue on them
      const int N = (int)c.h.N, D = (int)c.h.D;
      k_col_index<T><<<cdiv(N, kIndexWarps), 32 * kIndexWarps, 0, c.st>>>(R, 0, D, N, c.rmask.p, c.ccnt.p,
                                                                          c.clist.p);
      post_launch(c);
      // with the active set (the CG's product), warps whose outputs are all
      // masked by the epilogue skip their sums
      k_trans_col<T><<<dim3(cdiv(N, kTcWarps), cdiv(M, 32)), dim3(32, kTcWarps), 0, c.st>>>(
          M, N, D, c.ftile.p, c.ftile_lo.p, c.ftile_hi.p, c.ftile_off.p, R, c.rmask.p, c.ccnt.p, c.clist.p, G, pred,
          c.count_fmas ? c.fmacount.p + 1 : nullptr, ik, reduced ? c.maxr.p : nullptr);
      post_launch(c);
      raw = 1;
    }
  }
  if (raw) {
  } else if (sh.rows && W == nullptr && c.t_contiguous && RB > 0) {
    const int threads = cdiv((int64_t)RB * c.h.N, 32) * 32;
    k_trans_rows<T, HVP><<<cdiv(M, RB), threads, 0, c.st>>>(bd, tv, RB, R, V, rs, c.maxr.p, reduced, c2gam, ik, G,
                                                            pred, Gf);
    post_launch(c);
    return;
  }
  switch (sh.C) {
    case 1:
      k_trans<T, HVP, 1><<<M, sh.threads, 0, c.st>>>(bd, tv, R, V, rs, c.maxr.p, reduced, c2gam, ik, G, W, dpart, pred, Gf,
                                                      raw);
      break;
    case 2:
      k_trans<T, HVP, 2><<<M, sh.threads, 0, c.st>>>(bd, tv, R, V, rs, c.maxr.p, reduced, c2gam, ik, G, W, dpart, pred, Gf,
                                                      raw);
      break;
    case 4:
      k_trans<T, HVP, 4><<<M, sh.threads, 0, c.st>>>(bd, tv, R, V, rs, c.maxr.p, reduced, c2gam, ik, G, W, dpart, pred, Gf,
                                                      raw);
      break;
    default:
      k_trans<T, HVP, 8><<<M, sh.threads, 0, c.st>>>(bd, tv, R, V, rs, c.maxr.p, reduced, c2gam, ik, G, W, dpart, pred, Gf,
                                                      raw);
      break;
  }
  post_launch(c);
}

// k_trans with the context's schedule.
template <typename T, bool HVP>
static void launch_trans(Ctx& c, const T* tv, const T* R, const T* V, const T* rs, int reduced, T c2gam,
                         const int8_t* ik, T* G, const T* W, double* dpart, const double* pred, T* Gf = nullptr) {
  TransShape sh = c.sched.trans_threads > 0 ? TransShape{c.sched.trans_threads, c.sched.trans_cols}
                                            : trans_shape((int)c.h.N);
  sh.rows = c.sched.trans_rows;
  launch_trans_shape<T, HVP>(c, sh, tv, R, V, rs, reduced, c2gam, ik, G, W, dpart, pred, Gf);
}

// dL(X) -> c.G (975-1032), reusing R and the gradient itself when X and the
// space have not changed since they were computed (bitwise the same values).
static void op_dL(Ctx& c) {
  Scope s(c.timers, "dL");
  const int M = (int)c.h.M, N = (int)c.h.N;
  if (!c.fullspace) rebuild_x(c);
  if (c.G_ver == c.xver && c.G_full == c.fullspace) return;
  if (!c.exact && c.Gf_ver == c.xver) {
    // mixed path: the full-space gradient of this X is known
    if (c.fullspace) {
      CK(cudaMemcpyAsync(c.G.p, c.Gf.p, (size_t)M * N * 8, cudaMemcpyDeviceToDevice, c.st));
    } else {
      k_reduced_from_full<<<M, std::min(256, std::max(32, cdiv(N, 32) * 32)), 0, c.st>>>(c.Gf.p, c.maxr.p, N, c.G.p);
      post_launch(c);
    }
  } else if (c.df_trans) {
    // mixed path, double-FP32: full-space gradient into Gf (and G), then
    // the reduced one from it
    ensure_R(c);
    const int D = (int)c.h.D;
    k_split_df<<<elem_grid((int64_t)D * N), 256, 0, c.st>>>(c.R.p, (int64_t)D * N, 1.0, c.rdf.p);
    post_launch(c);
    double* g = c.fullspace ? c.G.p : nullptr;
    const double c2g = 2.0 * c.h.gam;
    const int rb = df_rows_per_block(M, N, c.df_rows, c.num_sms);
    const int threads = 32 * std::min(kDfColWarps, cdiv(N, 32));
    const dim3 grid(cdiv(M, rb), cdiv(N, threads));
    DevBands bd = bands_of(c);
    if (rb == 8) k_trans_df<8><<<grid, threads, 0, c.st>>>(bd, c.tdf.p, c.rdf.p, c.X.p, c2g, g, c.Gf.p);
    else if (rb == 4) k_trans_df<4><<<grid, threads, 0, c.st>>>(bd, c.tdf.p, c.rdf.p, c.X.p, c2g, g, c.Gf.p);
    else k_trans_df<2><<<grid, threads, 0, c.st>>>(bd, c.tdf.p, c.rdf.p, c.X.p, c2g, g, c.Gf.p);
    post_launch(c);
    if (!c.fullspace) {
      k_reduced_from_full<<<M, std::min(256, std::max(32, cdiv(N, 32) * 32)), 0, c.st>>>(c.Gf.p, c.maxr.p, N, c.G.p);
      post_launch(c);
    }
    c.Gf_ver = c.xver;
  } else {
    ensure_R(c);
    double* gf = (!c.exact && !c.fullspace) ? c.Gf.p : nullptr;
    launch_trans<double, false>(c, c.tval.p, c.R.p, c.X.p, nullptr, c.fullspace ? 0 : 1, 2.0 * c.h.gam, nullptr,
                                c.G.p, nullptr, nullptr, nullptr, gf);
    if (!c.exact) {
      if (c.fullspace) CK(cudaMemcpyAsync(c.Gf.p, c.G.p, (size_t)M * N * 8, cudaMemcpyDeviceToDevice, c.st));
      c.Gf_ver = c.xver;
    }
  }
  c.G_ver = c.xver;
  c.G_full = c.fullspace;
}

// pdot (589-614): sum(a.b) over M*N -> device scalar `out`.  FP64 path: one
// chain per column over the rows, columns added in ascending order.
static void dot_dev(Ctx& c, const double* a, const double* b, double* out, const double* pred = nullptr) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  if (c.exact) {
    // column chains, then (last block) their ascending sum into out
    k_colchain<0><<<dim3(cdiv(N, kChainWarps), 1), 32 * kChainWarps, 0, c.st>>>(a, b, 0, M, N, 0.0, c.colbuf.p,
                                                                                nullptr, pred, out, 1, c.counters.p + 2);
    post_launch(c);
    return;
  }
  const int64_t total = (int64_t)M * N;
  const int g = elem_grid(total);
  k_dot_part<<<g, 256, 0, c.st>>>(total, a, b, c.part.p);
  post_launch(c);
  reduce_to(c, c.part.p, g, out, 1, false, 0.0, pred);
}

// Two pdots of the FP64 CG at once: a.b -> out_ab, a.a -> out_aa, where
// out_aa = out_ab + ostride (a warp per chain, two per column).
static void dot2_exact(Ctx& c, const double* a, const double* b, double* out_ab, int ostride,
                       const double* pred) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  k_colchain<2><<<dim3(cdiv(N, kChainWarps / 2), 1), 32 * kChainWarps, 0, c.st>>>(
      a, b, 0, M, N, 0.0, c.colbuf.p, c.colbuf.p + N, pred, out_ab, ostride, c.counters.p + 3);
  post_launch(c);
}

// Hessian-vector product of one precision: Hp = H p (BF, 246-342); masks the
// active set and reduces p.Hp into sc[SC_V2] when ik != null.  `pred`
// points at the CG done flag (null: always run).
template <typename T>
static void hvp(Ctx& c, CGBufs<T>& b, const T* fv, const T* tv, const int8_t* ik, bool with_dot,
                const double* pred = nullptr) {
  const int M = (int)c.h.M;
  const T* src = c.fullspace ? b.p.p : b.V.p;
  {
    Scope sf(c.timers, "BF.fwd", true);
    launch_fwd<T, 1>(c, fv, src, 0, nullptr, b.R2.p, 1, pred);
  }
  Scope st(c.timers, "BF.trans", true);
  launch_trans<T, true>(c, tv, b.R2.p, b.p.p, c.fullspace ? nullptr : b.rs.p, c.fullspace ? 0 : 1,
                        (T)(2.0 * c.h.gam), ik, b.Hp.p, with_dot ? b.p.p : nullptr, with_dot ? c.part.p : nullptr,
                        pred);
  if (with_dot) reduce_to(c, c.part.p, M, c.sc.p + SC_V2, 1, false, 0.0, pred);
}

// ---------------------------------------------------------------------------
// Tensor-core (tcgen05 + TMA, split-BF16x3) Hessian products of the mixed CG.
// ---------------------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled from the driver (no link-time libcuda dependency).
static EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  if (!fn) throw Err(PQDTS_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  return fn;
}

// 2-D bf16 map: inner x outer elements, rows row_bytes apart, box
// box_inner x box_outer (box_inner * 2 = the stage row width kTcRowBytes,
// swizzled to match), zero fill outside the extents.
static void make_map_bf16(CUtensorMap* m, const void* base, uint64_t inner, uint64_t outer, uint64_t row_bytes,
                          uint32_t box_inner, uint32_t box_outer) {
  const cuuint64_t dims[2] = {inner, outer};
  const cuuint64_t strides[1] = {row_bytes};
  const cuuint32_t box[2] = {box_inner, box_outer};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = encode_tiled()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box,
                                    es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                    kTcRowBytes == 128  ? CU_TENSOR_MAP_SWIZZLE_128B
                                    : kTcRowBytes == 64 ? CU_TENSOR_MAP_SWIZZLE_64B
                                                        : CU_TENSOR_MAP_SWIZZLE_32B,
                                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Err(PQDTS_E_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

// Band rows (lo / w / off / val over R rows, FP64) as a TcOperand: values
// split into bf16 hi + lo (hi = bf16(v), lo = bf16(v - hi)).
static void build_tc_operand(Ctx& c, const std::vector<int32_t>& lo, const std::vector<int32_t>& w,
                             const std::vector<int64_t>& off, const std::vector<double>& val, int64_t R,
                             TcOperand& op) {
  const int blocks = cdiv(R, kTcRows);
  std::vector<int32_t> kb(blocks, -1), nch(blocks, 0);
  int kmax = kTcK;
  for (int b = 0; b < blocks; ++b) {
    int64_t k0 = INT64_MAX, k1 = -1;
    const int64_t r1 = std::min<int64_t>(R, (int64_t)(b + 1) * kTcRows);
    for (int64_t r = (int64_t)b * kTcRows; r < r1; ++r)
      if (w[r] > 0) {
        k0 = std::min<int64_t>(k0, lo[r]);
        k1 = std::max<int64_t>(k1, (int64_t)lo[r] + w[r]);
      }
    if (k1 < 0) continue;
    kb[b] = (int32_t)(k0 / kTcK * kTcK);
    nch[b] = (int32_t)((k1 - kb[b] + kTcK - 1) / kTcK);
    kmax = std::max(kmax, nch[b] * kTcK);
  }
  const size_t total = (size_t)blocks * kTcRows * kmax;
  std::vector<__nv_bfloat16> hv(total, __float2bfloat16(0.0f)), lv(total, __float2bfloat16(0.0f));
  for (int64_t r = 0; r < R; ++r) {
    const int b = (int)(r / kTcRows);
    for (int k = 0; k < w[r]; ++k) {
      const size_t x = (size_t)r * kmax + (size_t)(lo[r] + k - kb[b]);
      const double v = val[off[r] + k];
      const __nv_bfloat16 h = __double2bfloat16(v);
      hv[x] = h;
      lv[x] = __double2bfloat16(v - (double)__bfloat162float(h));
    }
  }
  op.hi.upload(hv.data(), total, c.st, &c.h2d);
  op.lo.upload(lv.data(), total, c.st, &c.h2d);
  op.kb.upload(kb.data(), blocks, c.st, &c.h2d);
  op.nch.upload(nch.data(), blocks, c.st, &c.h2d);
  op.h_nch = nch;
  op.scheds.clear();
  op.blocks = blocks;
  op.kmax = kmax;
  make_map_bf16(&op.map_hi, op.hi.p, kmax, (uint64_t)blocks * kTcRows, (uint64_t)kmax * 2, kTcK, kTcRows);
  make_map_bf16(&op.map_lo, op.lo.p, kmax, (uint64_t)blocks * kTcRows, (uint64_t)kmax * 2, kTcK, kTcRows);
  CK(cudaStreamSynchronize(c.st));  // the host staging vectors go out of scope
}

// Tile width over N: N split in mult * ceil(N/256) equal tiles, rounded up
// to 16 (MMA N for M = 128: 16..256 in steps of 16).
static int tc_tile_n(int64_t N, int mult) {
  const int64_t nt = (N + 255) / 256 * mult;
  const int64_t bn = ((N + nt - 1) / nt + 15) / 16 * 16;
  return (int)std::max<int64_t>(16, std::min<int64_t>(256, bn));
}

static uint32_t tc_stage_bytes(int bn) { return 2u * kTcRows * kTcRowBytes + 2u * (uint32_t)bn * kTcRowBytes; }
constexpr uint32_t kTcRing = 200u * 1024u;           // stage ring budget
constexpr uint32_t kTcMaxSmem = kTcRing + 1024u;      // + alignment slack

// Tile width BN of the tensor-core products: the B operands' maps (box
// 64 x BN) and the stage count follow it.
static void tc_configure(Ctx& c, int bn) {
  const int64_t M = c.h.M, N = c.h.N, D = c.h.D;
  const int stages = std::min<int>(kTcMaxStages, (int)(kTcRing / tc_stage_bytes(bn)));
  if (stages < 2) throw Err(PQDTS_E_STATE, "internal: tensor-core stage ring does not fit");
  // k_tc_band's FP32 epilogue stages the 128 x BN tile (rows padded to an odd
  // word count) in the ring
  const uint32_t staging = 128u * (uint32_t)(bn + ((33 - bn % 32) % 32)) * 4u;
  if ((uint32_t)stages * tc_stage_bytes(bn) < staging)
    throw Err(PQDTS_E_STATE, "internal: tensor-core epilogue staging does not fit the stage ring");
  make_map_bf16(&c.map_vt_hi, c.vt_hi.p, M, N, (uint64_t)c.tc_mp * 2, kTcK, bn);
  make_map_bf16(&c.map_vt_lo, c.vt_lo.p, M, N, (uint64_t)c.tc_mp * 2, kTcK, bn);
  make_map_bf16(&c.map_yt_hi, c.yt_hi.p, D, N, (uint64_t)c.tc_dp * 2, kTcK, bn);
  make_map_bf16(&c.map_yt_lo, c.yt_lo.p, D, N, (uint64_t)c.tc_dp * 2, kTcK, bn);
  c.tc_bn = bn;
  c.tc_stages = stages;
}

// Operands and maps of the tensor-core products (mixed precision, when the
// option allows and the device is a tcgen05 part).
static void setup_tc(Ctx& c) {
  c.tc_ready = false;
  if (c.precision != PQDTS_MIXED || c.tc_option == 0) return;
  int major = 0;
  CK(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, c.device));
  if (major != 10) {
    if (c.tc_option == 1) throw Err(PQDTS_E_ARG, "tensor-core products need a compute capability 10.x device");
    return;
  }
  const HostProblem& h = c.h;
  const int64_t M = h.M, N = h.N, D = h.D;
  const int bn = tc_tile_n(N, 1);
  build_tc_operand(c, h.flo, h.fw, h.foff, h.fval, D, c.tcF);
  build_tc_operand(c, h.tlo, h.tw, h.toff, h.tbval, M, c.tcFt);
  c.tc_mp = (M + 7) / 8 * 8;
  c.tc_dp = (D + 7) / 8 * 8;
  c.vt_hi.alloc((size_t)N * c.tc_mp);
  c.vt_lo.alloc((size_t)N * c.tc_mp);
  c.yt_hi.alloc((size_t)N * c.tc_dp);
  c.yt_lo.alloc((size_t)N * c.tc_dp);
  CK(cudaFuncSetAttribute(k_tc_band, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcMaxSmem));
  CK(cudaFuncSetAttribute(k_tc_band_p, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcMaxSmem));
  CK(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, c.device));
  tc_configure(c, bn);
  c.tc_ready = true;
}

// Tile lists of the persistent kernel for A's row blocks at N tile width bn
// and K splits `splits`: tiles (N tile fastest, then row block, then split)
// sorted by their K chunks, longest first, each given to the CTA with the
// least work so far (+2 chunks of fixed cost per tile); built once per
// problem and shape, outside any stream capture.
static TcSched& tc_sched(Ctx& c, TcOperand& A, int bn, int splits, int N = -1) {
  if (N < 0) N = (int)c.h.N;
  const std::array<int, 3> key{bn, splits, N};
  auto it = A.scheds.find(key);
  if (it != A.scheds.end()) return *it->second;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(c.st, &cs));
  if (cs != cudaStreamCaptureStatusNone) throw Err(PQDTS_E_STATE, "internal: tensor-core tile lists built in a capture");
  const int ntn = cdiv(N, bn);
  const int64_t T = (int64_t)ntn * A.blocks * splits;
  const int grid = (int)std::min<int64_t>(T, c.num_sms);
  std::vector<std::pair<int, int32_t>> cost((size_t)T);
  for (int64_t t = 0; t < T; ++t) {
    const int64_t rest = t / ntn;
    const int blk = (int)(rest % A.blocks), sp = (int)(rest / A.blocks);
    const int c1 = A.h_nch[blk], per = (c1 + splits - 1) / splits;
    const int s0 = std::min(c1, sp * per), s1 = std::min(c1, s0 + per);
    cost[t] = {s1 - s0 + 2, (int32_t)t};
  }
  std::stable_sort(cost.begin(), cost.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
  std::vector<std::vector<int32_t>> lists(grid);
  std::vector<int64_t> load(grid, 0);
  for (const auto& ct : cost) {
    const int g = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[g] += ct.first;
    lists[g].push_back(ct.second);
  }
  std::vector<int32_t> off(grid + 1, 0), tiles;
  tiles.reserve((size_t)T);
  for (int g = 0; g < grid; ++g) {
    // each CTA walks its tiles in tile order (N tiles of a row block together)
    std::sort(lists[g].begin(), lists[g].end());
    tiles.insert(tiles.end(), lists[g].begin(), lists[g].end());
    off[g + 1] = (int32_t)tiles.size();
  }
  auto sc = std::make_unique<TcSched>();
  sc->off.upload(off.data(), off.size(), c.st, &c.h2d);
  sc->tile.upload(tiles.data(), tiles.size(), c.st, &c.h2d);
  sc->grid = grid;
  CK(cudaStreamSynchronize(c.st));  // the host vectors go out of scope
  return *A.scheds.emplace(key, std::move(sc)).first->second;
}

// Out = scale * A . B^T on the tensor cores (A a TcOperand of R rows; B the
// K-major split operand behind bhi / blo, Nw rows: the problem's N unless
// given); mode 0: FP32 partials (splits of the K range, out_stride apart),
// mode 1: transposed bf16 split into oh / ol.
static void tc_product(Ctx& c, TcOperand& A, const CUtensorMap& bhi, const CUtensorMap& blo, int R, int splits,
                       int mode, float scale, float* out, __nv_bfloat16* oh, __nv_bfloat16* ol, int64_t ld,
                       const double* pred, int persistent, int Nw = -1) {
  const int N = Nw > 0 ? Nw : (int)c.h.N;
  const size_t smem = (size_t)c.tc_stages * tc_stage_bytes(c.tc_bn) + 1024;
  if (persistent) {
    TcSched& ts = tc_sched(c, A, c.tc_bn, splits, N);
    k_tc_band_p<<<ts.grid, kTcpThreads, smem, c.st>>>(A.map_hi, A.map_lo, bhi, blo, A.kb.p, A.nch.p, R, N, c.tc_bn,
                                                      c.tc_stages, splits, A.blocks, mode, scale, out, (int64_t)R * N,
                                                      oh, ol, ld, pred, c.sc.p + SC_TCERR, c.tc_wait_ns,
                                                      c.tc_wait_probe, ts.off.p, ts.tile.p);
  } else {
    const dim3 grid(cdiv(N, c.tc_bn), A.blocks, splits);
    k_tc_band<<<grid, kTcThreads, smem, c.st>>>(A.map_hi, A.map_lo, bhi, blo, A.kb.p, A.nch.p, R, N, c.tc_bn,
                                                c.tc_stages, splits, mode, scale, out, (int64_t)R * N, oh, ol, ld, pred,
                                                c.sc.p + SC_TCERR, c.tc_wait_ns, c.tc_wait_probe);
  }
  post_launch(c);
}

// F.V on the tensor cores into the (2 F.V)^T split operand: directly from
// the epilogue, or (splits1 > 1) through FP32 partials of its K segments.
static void tc_forward(Ctx& c, int splits1, int persistent, const double* pred) {
  const int N = (int)c.h.N, D = (int)c.h.D;
  if (splits1 <= 1) {
    tc_product(c, c.tcF, c.map_vt_hi, c.map_vt_lo, D, 1, 1, 2.0f, nullptr, c.yt_hi.p, c.yt_lo.p, c.tc_dp, pred,
               persistent);
    return;
  }
  require(c.ypart.p, "F.V partials");
  tc_product(c, c.tcF, c.map_vt_hi, c.map_vt_lo, D, splits1, 0, 2.0f, c.ypart.p, nullptr, nullptr, 0, pred,
             persistent);
  k_finish_t<<<dim3(cdiv(D, 32), cdiv(N, 32)), dim3(32, 8), 0, c.st>>>(c.ypart.p, splits1, D, N, c.tc_dp, c.yt_hi.p,
                                                                       c.yt_lo.p, pred);
  post_launch(c);
}

// The Hessian product pair on the tensor cores: V -> V^T split, then
// (2 F.V)^T split (written by the first product's epilogue), then the
// partials of F^T.(2 F.V) in hpart32 (tc_splits of them).
static void tc_hvp_products(Ctx& c, const float* src, const double* pred, bool presplit) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  if (!presplit) {
    k_split_t<<<dim3(cdiv(M, 32), cdiv(N, 32)), dim3(32, 8), 0, c.st>>>(src, M, N, c.tc_mp, c.vt_hi.p, c.vt_lo.p,
                                                                         pred);
    post_launch(c);
  }
  {
    Scope sd(c.timers, "CG.tc_fwd", true);
    tc_forward(c, c.sched.tc_splits1, c.sched.tc_persistent, pred);
  }
  Scope sd(c.timers, "CG.tc_trans", true);
  tc_product(c, c.tcFt, c.map_yt_hi, c.map_yt_lo, M, c.sched.tc_splits, 0, 1.0f, c.hpart32.p, nullptr, nullptr, 0,
             pred, c.sched.tc_persistent);
}

// The line-search probes' split operand and its maps (allocated on first
// use, zero filled: rows beyond nb * N feed only columns that are never
// stored; maps rebuilt when the tile width, buffer or stride changed).
static void ensure_ls_operand(Ctx& c) {
  const int64_t rows = (int64_t)kBatchLS * c.h.N;
  const size_t need = (size_t)rows * (size_t)c.tc_mp;
  if (c.ls_hi.p == nullptr || c.ls_hi.cap < need) {
    c.ls_hi.alloc(need);
    c.ls_lo.alloc(need);
    CK(cudaMemsetAsync(c.ls_hi.p, 0, need * sizeof(__nv_bfloat16), c.st));
    CK(cudaMemsetAsync(c.ls_lo.p, 0, need * sizeof(__nv_bfloat16), c.st));
  }
  if (c.ls_map_bn != c.tc_bn || c.ls_map_ptr != c.ls_hi.p || c.ls_map_mp != c.tc_mp || c.ls_map_rows != rows) {
    make_map_bf16(&c.map_ls_hi, c.ls_hi.p, c.h.M, rows, (uint64_t)c.tc_mp * 2, kTcK, c.tc_bn);
    make_map_bf16(&c.map_ls_lo, c.ls_lo.p, c.h.M, rows, (uint64_t)c.tc_mp * 2, kTcK, c.tc_bn);
    c.ls_map_bn = c.tc_bn;
    c.ls_map_ptr = c.ls_hi.p;
    c.ls_map_mp = c.tc_mp;
    c.ls_map_rows = rows;
  }
}

// F.dX of nb line-search probes (Xc[0..nb) against X0) on the tensor cores:
// one product over the probes' N' = nb * N columns into fdx32 (D x N'
// row-major FP32; probe b's columns b * N ..).
static void tc_probe_products(Ctx& c, const double* Xc, const double* X0, int nb) {
  const int M = (int)c.h.M, N = (int)c.h.N, D = (int)c.h.D;
  ensure_ls_operand(c);
  k_delta_split_t<<<dim3(cdiv(M, 32), cdiv(N, 32), nb), dim3(32, 8), 0, c.st>>>(Xc, X0, M, N, c.tc_mp, c.ls_hi.p,
                                                                               c.ls_lo.p);
  post_launch(c);
  tc_product(c, c.tcF, c.map_ls_hi, c.map_ls_lo, D, 1, 0, 1.0f, c.fdx32.p, nullptr, nullptr, 0, nullptr,
             c.sched.tc_persistent, nb * N);
}

// Out (R x N) = scale * Band (R rows) . In with tile code `tile` (0 = 64x64,
// 1 = 64x32, 2 = 32x32 rows x columns); grid.z = nz stacked products
// (in_stride / out_stride apart) or, with splits > 1, the K segments of one
// product (partials out_stride apart, summed by the consumer).
static void launch_band_gemm32(Ctx& c, int tile, const int32_t* lo, const int32_t* w, const int64_t* off,
                               const float* vals, const float* In, int R, int N, float scale, float* Out,
                               const double* pred, int nz = 1, int64_t in_stride = 0, int64_t out_stride = 0,
                               int splits = 1) {
  switch (tile) {
    case 0:
      k_band_gemm32<64, 64><<<dim3(cdiv(N, 64), cdiv(R, 64), nz), 256, 0, c.st>>>(lo, w, off, vals, In, R, N, scale,
                                                                                   Out, pred, in_stride, out_stride,
                                                                                   splits);
      break;
    case 1:
      k_band_gemm32<64, 32><<<dim3(cdiv(N, 32), cdiv(R, 64), nz), 128, 0, c.st>>>(lo, w, off, vals, In, R, N, scale,
                                                                                   Out, pred, in_stride, out_stride,
                                                                                   splits);
      break;
    default:
      k_band_gemm32<32, 32><<<dim3(cdiv(N, 32), cdiv(R, 32), nz), 64, 0, c.st>>>(lo, w, off, vals, In, R, N, scale,
                                                                                 Out, pred, in_stride, out_stride,
                                                                                 splits);
      break;
  }
  post_launch(c);
}

// CTAs of a tile code over an R x N output.
static int64_t tile_ctas(int tile, int R, int N) {
  const int tr = tile == 2 ? 32 : 64, tn = tile == 0 ? 64 : 32;
  return (int64_t)cdiv(R, tr) * cdiv(N, tn);
}

// Heuristic tile: the largest that still gives two CTAs per SM (small
// problems need more, smaller tiles to fill the GPU).
static int heuristic_tile(int R, int N, int nz = 1) {
  const int64_t want = 2 * 152;
  if (tile_ctas(0, R, N) * nz >= want) return 0;
  if (tile_ctas(1, R, N) * nz >= want) return 1;
  return 2;
}

// Rows per block of the multi-row Hessian epilogue: about four blocks per
// SM over the M rows, at most kEpiMaxRows.
static int epi_rows(const Ctx& c, int64_t M) {
  const int64_t want = M / std::max<int64_t>(1, 4 * (c.num_sms > 0 ? c.num_sms : 152));
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, kEpiMaxRows));
}
constexpr int kEpiThreads = 256;

// The FP32 Hessian row epilogue over hpart32's `parts` partials (several
// rows per block, streaming); returns the number of p.Hp partials written,
// or 0 when the multi-row form has already summed them into *vsum (its
// last block, vsum != null).
static int hvp_epilogue(Ctx& c, const float* p, const float* rs, const int8_t* ik, float* Hp, double* dpart,
                        const double* pred, int parts, double* vsum = nullptr) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  const int RB = epi_rows(c, M);
  if (c.rows_option != 0) {
    const bool fused = vsum != nullptr && dpart != nullptr;
    k_hvp_epi32_rows<<<cdiv(M, RB), kEpiThreads, 0, c.st>>>(c.hpart32.p, p, rs, c.maxr.p, rs ? 1 : 0,
                                                            (float)(2.0 * c.h.gam), ik, M, N, RB, Hp, dpart, pred,
                                                            parts, fused ? vsum : nullptr,
                                                            fused ? c.counters.p + 4 : nullptr);
    post_launch(c);
    return fused ? 0 : cdiv(M, RB);
  }
  const int tb = std::min(256, std::max(32, cdiv(N, 32) * 32));
  k_hvp_epi32<<<M, tb, 0, c.st>>>(c.hpart32.p, p, rs, c.maxr.p, rs ? 1 : 0, (float)(2.0 * c.h.gam), ik, M, N, Hp,
                                  dpart, pred, parts);
  post_launch(c);
  return M;
}

// Mixed precision Hessian product Hp = H p in FP32 with the tiled band
// products (F.V then F^T.(2O)) and the row epilogue; p.Hp -> sc[SC_V2].
// presplit: V's transposed split is already in place (k_lift_split32).
static void hvp32(Ctx& c, CGBufs<float>& b, const int8_t* ik, bool with_dot, const double* pred,
                  bool presplit = false) {
  const int M = (int)c.h.M, N = (int)c.h.N, D = (int)c.h.D;
  const float* src = c.fullspace ? b.p.p : b.V.p;
  require(c.hpart32.p, "split-K partials");
  int parts;
  if (c.sched.tc) {
    tc_hvp_products(c, src, pred, presplit);
    parts = c.sched.tc_splits;
  } else {
    launch_band_gemm32(c, c.sched.fwd_tile, c.flo.p, c.fw.p, c.foff.p, c.fval32.p, src, D, N, 2.0f, b.R2.p, pred);
    // F^T.(2O) with its K range split in trn_splits segments; the epilogue
    // sums the partial products in a fixed order
    parts = c.sched.trn_splits;
    launch_band_gemm32(c, c.sched.trn_tile, c.tlo.p, c.tw.p, c.toff.p, c.tbval32.p, b.R2.p, M, N, 1.0f, c.hpart32.p,
                       pred, parts, 0, (int64_t)M * N, parts);
  }
  Scope sd(c.timers, "CG.epilogue", true);
  const int nparts = hvp_epilogue(c, b.p.p, c.fullspace ? nullptr : b.rs.p, ik, b.Hp.p, with_dot ? c.part.p : nullptr,
                                  pred, parts, with_dot ? c.sc.p + SC_V2 : nullptr);
  if (with_dot && nparts > 0) reduce_to(c, c.part.p, nparts, c.sc.p + SC_V2, 1, false, 0.0, pred);
}

// A chunk of CG iterations captured as a CUDA graph (on first use of its
// key: variant, space, constants; every kernel of it reads the context's
// fixed buffers, so a replay is the same launches).
template <class Body>
static CGGraph& captured(Ctx& c, const std::array<uint64_t, 5>& key, int spans, Body&& body) {
  auto it = c.graphs.find(key);
  if (it != c.graphs.end()) return it->second;
  CGGraph g;
  for (int k = 0; k < 2 * spans; ++k) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    c.timers.capture_pool.push_back(e);
  }
  const int64_t l0 = c.launches;
  cudaGraph_t graph = nullptr;
  CK(cudaStreamBeginCapture(c.st, cudaStreamCaptureModeThreadLocal));
  c.timers.capture = &g.spans;
  try {
    body();
  } catch (...) {
    c.timers.capture = nullptr;
    cudaStreamEndCapture(c.st, &graph);
    if (graph) cudaGraphDestroy(graph);
    c.launches = l0;
    g.destroy();
    throw;
  }
  c.timers.capture = nullptr;
  const cudaError_t e = cudaStreamEndCapture(c.st, &graph);
  g.kernels = c.launches - l0;
  c.launches = l0;  // nothing ran yet: replays are counted
  if (e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    g.destroy();
    CK(e);
  }
  const cudaError_t e2 = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e2 != cudaSuccess) {
    g.destroy();
    CK(e2);
  }
  return c.graphs.emplace(key, g).first->second;
}

// Queues CG iterations in chunks (4, then 8) and polls the exit flag after
// each chunk; iterations queued after the exit are no-ops (each kernel reads
// the flag first), the flag is also set at the iteration limit.  With graphs
// on, a chunk is one replay of a captured graph.  Returns the iterations run.
template <class Iter>
static int cg_chunks(Ctx& c, std::array<uint64_t, 4> variant, Iter&& iteration) {
  int queued = 0;
  for (int chunk_no = 0;; ++chunk_no) {
    const bool first = chunk_no == 0;
    const int chunk = first ? 4 : 8;
    if (c.use_graphs) {
      const int spans = chunk * (c.timers.detail ? 8 : 1);  // timer spans recorded per chunk
      CGGraph& gr = captured(c, {variant[0], variant[1], variant[2], variant[3], (uint64_t)first}, spans, [&] {
        for (int k = 0; k < chunk; ++k) iteration(first && k == 0);
      });
      CK(cudaGraphLaunch(gr.exec, c.st));
      c.launches += gr.kernels;
      queued += chunk;
      read_back(c, c.sc.p, SC_NSC);
      c.timers.harvest(gr.spans);
    } else {
      for (int k = 0; k < chunk && queued < kMaxCG; ++k, ++queued) iteration(queued == 0);
      read_back(c, c.sc.p, SC_NSC);
    }
    check_tc_error(c);
    if (c.pin[SC_DONE] != 0.0 || queued >= kMaxCG) return (int)c.pin[SC_ITER];
  }
}

// The truncated-Newton PCG (2007-2090) in FP32 (mixed precision): the same
// recurrence and exit test as cg_solve, tiled FP32 products, warp-per-row
// lift, FP32 vectors with FP64 block sums.
// The FP32 CG's start (2007-2035): active set, r = -g, z, p, sn = 0, the
// forcing term's scalars and the FP32 preconditioner.
static void cg32_begin(Ctx& c, double bdfac) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  const int64_t MN = (int64_t)M * N;
  const int g = elem_grid(MN);
  CGBufs<float>& b = c.cg32;
  require(c.tbval32.p, "F^T band values (FP32)");
  k_rsqrt_diag<<<cdiv(M, 256), 256, 0, c.st>>>(c.bdiag.p, bdfac, M, c.rsq32.p);
  post_launch(c);
  k_cg_init32<<<g, 256, 0, c.st>>>(c.X.p, c.G.p, c.rsq32.p, kActiveTol, M, N, c.ik.p, b.r.p, b.z.p, b.p.p, b.sn.p,
                                   c.part.p, c.part2.p, c.ipart.p);
  post_launch(c);
  reduce_to(c, c.part.p, g, c.sc.p + SC_NORM);
  reduce_to(c, c.part2.p, g, c.sc.p + SC_RZ);
  k_sum_i<<<1, 256, 0, c.st>>>(c.ipart.p, g, c.icount.p);
  post_launch(c);
  k_cg_scalars0<<<1, 1, 0, c.st>>>(c.sc.p);
  post_launch(c);
  if (c.verbose) {
    long long nact = 0;
    CK(cudaMemcpyAsync(&nact, c.icount.p, sizeof(long long), cudaMemcpyDeviceToHost, c.st));
    CK(cudaStreamSynchronize(c.st));
    ListLine l;
    l.s("positivity constraints").i8(nact).s("active of").i8(MN).r8((double)nact / (double)MN).print();
  }
}

// The FP32 CG's end: its iteration count and (verbose) the reference's
// newton-pcg lines.
static void cg32_end(Ctx& c, int done_iters) {
  c.n_cg += done_iters;
  if (c.verbose) {
    std::vector<double> lg(4 * kMaxCG);
    CK(cudaMemcpyAsync(lg.data(), c.cglog.p, lg.size() * 8, cudaMemcpyDeviceToHost, c.st));
    CK(cudaStreamSynchronize(c.st));
    for (int j = 0; j < done_iters; ++j) {
      ListLine l;
      l.s("newton-pcg").i4(j + 1).s("sqrt(b2)=").r8(lg[4 * j]).s("eps=").r8(lg[4 * j + 1]).s("b1=").r8(lg[4 * j + 2]);
      l.s("v2=").r8(lg[4 * j + 3]).print();
    }
  }
}

static void cg_solve32(Ctx& c, double bdfac) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  const int64_t MN = (int64_t)M * N;
  const int g = elem_grid(MN);
  CGBufs<float>& b = c.cg32;
  Scope s(c.timers, "CG");
  cg32_begin(c, bdfac);
  const int lift_blocks = cdiv((int64_t)M * 32, 256);
  const int gs = std::min(g, cdiv(M, 8));  // the step's blocks: 8 warps, one row per warp
  const bool tc = c.sched.tc != 0;
  auto iteration = [&](bool first) {
    if (tc) {
      // p update, BF's lift (reduced space: row sums) and the first
      // product's operand split in one launch (no row-major V)
      Scope sd(c.timers, "CG.lift_split", true);
      k_cg_lift_split<32><<<cdiv(M, 32), dim3(32, 32), 0, c.st>>>(c.sc.p, first ? 0 : 1, M, N, b.p.p, b.z.p,
                                                              c.fullspace ? nullptr : c.maxr.p, b.rs.p, c.tc_mp,
                                                              c.vt_hi.p, c.vt_lo.p);
      post_launch(c);
    } else if (c.fullspace) {
      if (!first) {
        k_cg_pupdate<float><<<g, 256, 0, c.st>>>(c.sc.p, MN, b.p.p, b.z.p);
        post_launch(c);
      }
    } else {
      k_cg_lift32<<<lift_blocks, 256, 0, c.st>>>(first ? nullptr : c.sc.p, first ? 0 : 1, M, N, b.p.p, b.z.p,
                                                 c.maxr.p, b.V.p, b.rs.p);
      post_launch(c);
    }
    {
      Scope sb(c.timers, "BF");
      hvp32(c, b, c.ik.p, true, c.sc.p, tc);
    }
    // the step (one warp per row); its last block sums r.z, r.r and
    // advances the CG scalars
    Scope sd(c.timers, "CG.step", true);
    k_cg_step32<<<gs, 256, 0, c.st>>>(c.sc.p, c.rsq32.p, M, N, b.p.p, b.Hp.p, b.sn.p, b.r.p, b.z.p, c.part.p,
                                      c.part2.p, c.cglog.p, kMaxCG, c.counters.p + 1);
    post_launch(c);
  };
  const int done_iters = cg_chunks(c, {0, (uint64_t)c.fullspace, 0, 0}, iteration);
  cg32_end(c, done_iters);
}

// ---------------------------------------------------------------------------
// Truncated-Newton PCG (2007-2090) on device vectors of type T.
// ---------------------------------------------------------------------------
template <typename T>
static void cg_solve(Ctx& c, CGBufs<T>& b, const T* fv, const T* tv, double bdfac, int64_t* nact_out) {
  require(fv, "F values");
  require(tv, "F^T values");
  require(b.r.p, "CG vectors");
  const int M = (int)c.h.M, N = (int)c.h.N;
  const int64_t MN = (int64_t)M * N;
  const int g = elem_grid(MN);
  Scope s(c.timers, "CG");
  k_cg_init<T><<<g, 256, 0, c.st>>>(c.X.p, c.G.p, c.bdiag.p, bdfac, kActiveTol, M, N, c.ik.p, b.r.p, b.z.p, b.p.p,
                                    b.sn.p, c.part.p, c.part2.p, c.ipart.p);
  post_launch(c);
  k_sqrt_diag<<<cdiv(M, 256), 256, 0, c.st>>>(c.bdiag.p, bdfac, M, c.sqd.p);
  post_launch(c);
  constexpr bool kF64 = std::is_same<T, double>::value;
  const bool exact = kF64 && c.exact;
  if (exact) {
    if constexpr (kF64) {
      // r.z -> SC_RZ and r.r -> SC_NORM ((-g).(-g) == g.g bit for bit)
      static_assert(SC_NORM - SC_RZ == 3, "scalar layout");
      dot2_exact(c, b.r.p, b.z.p, c.sc.p + SC_RZ, SC_NORM - SC_RZ, nullptr);
    }
  } else {
    reduce_to(c, c.part.p, g, c.sc.p + SC_NORM);
    reduce_to(c, c.part2.p, g, c.sc.p + SC_RZ);
  }
  k_sum_i<<<1, 256, 0, c.st>>>(c.ipart.p, g, c.icount.p);
  post_launch(c);
  k_cg_scalars0<<<1, 1, 0, c.st>>>(c.sc.p);
  post_launch(c);
  if (c.verbose) {
    long long nact = 0;
    CK(cudaMemcpyAsync(&nact, c.icount.p, sizeof(long long), cudaMemcpyDeviceToHost, c.st));
    CK(cudaStreamSynchronize(c.st));
    if (nact_out) *nact_out = nact;
    ListLine l;
    l.s("positivity constraints").i8(nact).s("active of").i8(MN).r8((double)nact / (double)MN).print();
  }
  auto iteration = [&](bool first) {
    if (!first) {
      if (c.fullspace) {
        k_cg_pupdate<T><<<g, 256, 0, c.st>>>(c.sc.p, MN, b.p.p, b.z.p);
        post_launch(c);
      } else {
        k_cg_lift<T><<<cdiv(M, 32), kLiftThreads, 0, c.st>>>(c.sc.p, 1, M, N, b.p.p, b.z.p, c.maxr.p, b.V.p,
                                                                       b.rs.p);
        post_launch(c);
      }
    } else if (!c.fullspace) {
      k_cg_lift<T><<<cdiv(M, 32), kLiftThreads, 0, c.st>>>(nullptr, 0, M, N, b.p.p, b.z.p, c.maxr.p, b.V.p,
                                                                     b.rs.p);
      post_launch(c);
    }
    {
      Scope sb(c.timers, "BF");
      hvp<T>(c, b, fv, tv, c.ik.p, !exact, c.sc.p);
    }
    if constexpr (kF64)
      if (exact) dot_dev(c, b.p.p, b.Hp.p, c.sc.p + SC_V2, c.sc.p);
    k_cg_step<T><<<g, 256, 0, c.st>>>(c.sc.p, c.sqd.p, M, N, b.p.p, b.Hp.p, b.sn.p, b.r.p, b.z.p,
                                      exact ? nullptr : c.part.p, exact ? nullptr : c.part2.p);
    post_launch(c);
    if (exact) {
      if constexpr (kF64) {
        static_assert(SC_RR - SC_RZ == 1, "scalar layout");
        dot2_exact(c, b.r.p, b.z.p, c.sc.p + SC_RZ, 1, c.sc.p);
      }
    } else {
      reduce_to(c, c.part.p, g, c.sc.p + SC_RZ, 1, false, 0.0, c.sc.p);
      reduce_to(c, c.part2.p, g, c.sc.p + SC_RR, 1, false, 0.0, c.sc.p);
    }
    k_cg_scalars1<<<1, 1, 0, c.st>>>(c.sc.p, c.cglog.p, kMaxCG);
    post_launch(c);
  };
  uint64_t bdbits;
  std::memcpy(&bdbits, &bdfac, 8);
  const uint64_t kind = kF64 ? (exact ? 1 : 2) : 3;
  const int done_iters = cg_chunks(c, {kind, (uint64_t)c.fullspace, bdbits, 0}, iteration);
  c.n_cg += done_iters;
  if (c.verbose) {
    std::vector<double> lg(4 * kMaxCG);
    CK(cudaMemcpyAsync(lg.data(), c.cglog.p, lg.size() * 8, cudaMemcpyDeviceToHost, c.st));
    CK(cudaStreamSynchronize(c.st));
    for (int j = 0; j < done_iters; ++j) {
      ListLine l;
      l.s("newton-pcg").i4(j + 1).s("sqrt(b2)=").r8(lg[4 * j]).s("eps=").r8(lg[4 * j + 1]).s("b1=").r8(lg[4 * j + 2]);
      l.s("v2=").r8(lg[4 * j + 3]).print();
    }
  }
}

// Row-wise simplex projection (doproj, 1120-1140) of X + alpha_b*S (or of X
// when S is null) into out[b].  FP64 path: Condat's algorithm in the
// reference's order (bitwise equal to condat_simplexproj.c), one thread per
// row.  Mixed path: one warp per row, Michelot's fixed point.
static void project_rows(Ctx& c, const double* X, const double* S, const double* alphas, double* out, int B) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  const int64_t MN = (int64_t)M * N;
  if (c.exact) {
    const size_t smem = (size_t)2 * 33 * N * sizeof(double);
    if (smem <= kCondatSmemMax) {
      k_condat_smem<<<dim3(cdiv(M, 32), B), 32, smem, c.st>>>(X, S, alphas, out, MN, M, N);
    } else {
      require(c.aux.p, "aux");
      k_condat<<<dim3(cdiv(M, kRowThreads), B), kRowThreads, 0, c.st>>>(X, S, alphas, out, c.aux.p, MN, M, N);
    }
  } else {
    // rows staged in shared memory: up to 4 warps (rows) per block
    const int wpb = (int)std::min<int64_t>(4, (int64_t)kCondatSmemMax / ((int64_t)N * 8));
    if (wpb >= 1) {
      k_simplex_smem<<<dim3(cdiv(M, wpb), B), 32 * wpb, (size_t)wpb * N * sizeof(double), c.st>>>(X, S, alphas, out,
                                                                                                 MN, M, N);
    } else {
      k_simplex<<<dim3(cdiv((int64_t)M * 32, 128), B), 128, 0, c.st>>>(X, S, alphas, out, MN, M, N);
    }
  }
  post_launch(c);
}

// Candidates X + alpha_b*S (b < B) projected the way the stage requires and
// rebuilt as L does, their objectives and (stage 2) xmin into c.pin.
static void eval_candidates(Ctx& c, const double* al, int B, bool stage2, double* L, double* xmin) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  const int64_t MN = (int64_t)M * N;
  CK(cudaMemcpyAsync(c.alphas.p, al, B * sizeof(double), cudaMemcpyHostToDevice, c.st));
  if (stage2) {
    const int gb = cdiv(M, 32);  // 32-row tiles
    Scope s(c.timers, "doproj2");
    k_cand_proj2_t<<<dim3(gb, B), kTileThreads, 0, c.st>>>(c.X.p, c.sn64.p, c.alphas.p, c.Xc.p, MN, c.maxr.p, M, N, 1,
                                                         c.part2.p);
    post_launch(c);
    reduce_to(c, c.part2.p, gb, c.lsout.p + 2 * kBatchLS, B, true, 0.0);
  } else {
    Scope s(c.timers, "doproj");
    project_rows(c, c.X.p, c.sn64.p, c.alphas.p, c.Xc.p, B);
  }
  {
    Scope s(c.timers, "L");
    objective_stack(c, c.Xc.p, B);
  }
  fetch_objectives(c, B, L);
  for (int b = 0; b < B; ++b) xmin[b] = stage2 ? c.pin[2 * kBatchLS + b] : 0.0;
  c.n_lsL += B;
  // this batch stays in Xc / Rst until the next one: the mixed path adopts
  // the chosen candidate as the new iterate instead of recomputing it
  c.cand_xver = c.xver;
  c.cand_B = B;
  c.cand_stage2 = stage2;
  for (int b = 0; b < B; ++b) {
    c.cand_alpha[b] = al[b];
    c.cand_L[b] = L[b];
    c.cand_Lgam[b] = (c.h.gam != 0 && !c.exact) ? c.pin[kBatchLS + b] : 0.0;
    c.cand_xmin[b] = xmin[b];
  }
}

// Projected backtracking line search: Lalpha_min_auglag (440-483) in the
// full space, Lalpha_min2 (394-438) in the reduced space.  Step lengths are
// evaluated kBatchLS at a time; the reference's sequential accept rule is
// then applied to them in order, so the chosen alpha is the same.
// State of the reference's sequential backtracking (374-388, 420-435,
// 466-480): probes alpha_i = 0.75^(i-1), the smallest L seen (feasible in
// stage 2), stop at the first probe with sufficient decrease.
struct LSState {
  double L0, df, lm = kHuge, alphamin = 0.0, next_a = 1.0;
  int i = 1;  // index of the next probe
  bool done = false;
};

// One probe's decision; returns true when the search stops at it.
static bool ls_take(Ctx& c, LSState& ls, bool stage2, double alpha_i, double Lp, double xmin) {
  const bool better = stage2 ? (Lp < ls.lm && xmin >= -kFeasTol) : (Lp < ls.lm);
  if (better) {
    ls.lm = Lp;
    ls.alphamin = alpha_i;
  }
  if (c.verbose) {
    ListLine l;
    l.s("line search").i8(ls.i).s("L=").r8(Lp).s("alpha=").r8(alpha_i).s("df(0)=").r8(ls.df);
    if (stage2) l.s("min(X)=").r8(xmin);
    l.print();
  }
  ls.i++;
  const double armijo = std::fma(0.1 * alpha_i, ls.df, ls.L0);
  const bool shrink = stage2 ? (Lp > armijo || xmin < -kFeasTol) : (Lp > armijo);
  if (!shrink) ls.done = true;
  return ls.done;
}

// The rest of the sequence with FP64 objectives, first_batch probes at a
// time then doubling (the reference's rule applied to each batch in order).
static void ls_continue_fp64(Ctx& c, LSState& ls, bool stage2, int first_batch) {
  double qa[kBatchLS], qL[kBatchLS], qx[kBatchLS];
  int nb = first_batch;
  while (!ls.done && ls.i <= kMaxLS) {
    const int qlen = std::min(nb, kMaxLS - ls.i + 1);
    nb = std::min(kBatchLS, 2 * nb);
    for (int k = 0; k < qlen; ++k) {
      qa[k] = ls.next_a;
      ls.next_a = ls.next_a * 0.75;
    }
    eval_candidates(c, qa, qlen, stage2, qL, qx);
    for (int k = 0; k < qlen && !ls.done; ++k) ls_take(c, ls, stage2, qa[k], qL[k], qx[k]);
  }
}

// Projected backtracking line search: Lalpha_min_auglag (440-483) in the
// full space, Lalpha_min2 (394-438) in the reduced space.  FP64 path: every
// probe's objective in FP64, evaluated in batches (3, 2, 4, 8, ...), the
// reference's sequential rule applied to them in order -- the same alpha.
static void line_search(Ctx& c, bool stage2, double& alpha, double& dlalpha) {
  Scope s(c.timers, "Lalpha_min");
  double al[3] = {0.0, 0.0 + kDx, 1.0}, L[3], xm[3];
  eval_candidates(c, al, 3, stage2, L, xm);
  LSState ls;
  ls.L0 = L[0];
  ls.df = (L[1] - ls.L0) / kDx;
  dlalpha = ls.df;
  ls.next_a = 1.0 * 0.75;
  ls_take(c, ls, stage2, 1.0, L[2], xm[2]);
  ls_continue_fp64(c, ls, stage2, 2);
  alpha = ls.alphamin;
}

// Mixed path: the reference's probes (alpha = dx for the slope, then 1,
// 0.75, ...) are evaluated as objective changes relative to the alpha = 0
// candidate X0 (the iterate),
//   L(X_a) - L(X0) = sum F.dX (2 r0 + F.dX) + Lgam(X_a) - Lgam(X0),
// dX = X_a - X0 (projected), products in FP32 and sums in FP64 (the change
// itself to ~1e-6 relative, where a difference of FP32 objectives would be
// off by ~1e-2); the chosen step then gets an objective to FP64 accuracy
// (double-FP32 product unless that option is off, FP64 sums) and the
// sufficient-decrease check, and if it fails the reference's sequence
// continues from the next probe with such objectives.
static void line_search_mixed(Ctx& c, bool stage2, double& alpha, double& dlalpha) {
  Scope s(c.timers, "Lalpha_min");
  const int M = (int)c.h.M, N = (int)c.h.N, D = (int)c.h.D;
  const int64_t MN = (int64_t)M * N, DN = (int64_t)D * N;
  // alpha = 0: the projection of the (feasible) iterate is the iterate to
  // within ulps, so X, its objective and its residual R/2 serve as X0
  const double L0 = op_L(c);
  const double Lgam0 = c.Lgam_cache;
  ensure_R(c);
  CK(cudaMemcpyAsync(c.x0c.p, c.X.p, MN * sizeof(double), cudaMemcpyDeviceToDevice, c.st));
  k_half_to32<<<elem_grid(DN), 256, 0, c.st>>>(c.R.p, DN, 0.5f, c.r0_32.p);
  post_launch(c);
  const int g = elem_grid(MN), g2 = elem_grid(DN);
  const bool tc_screen = c.sched.tc && c.tc_ready && c.tc_screen_option != 0;
  // objective changes L(X_a) - L(X0) of nb projected probes -> dL[], xmin[]
  auto screen = [&](const double* qa, int nb, double* dL, double* xmin) {
    CK(cudaMemcpyAsync(c.alphas.p, qa, nb * sizeof(double), cudaMemcpyHostToDevice, c.st));
    if (stage2) {
      const int gb = cdiv(M, 32);  // 32-row tiles
      k_cand_proj2_t<<<dim3(gb, nb), kTileThreads, 0, c.st>>>(c.X.p, c.sn64.p, c.alphas.p, c.Xc.p, MN, c.maxr.p, M, N, 1,
                                                            c.part2.p);
      post_launch(c);
      reduce_to(c, c.part2.p, gb, c.lsout.p + 2 * kBatchLS, nb, true, 0.0);
    } else {
      project_rows(c, c.X.p, c.sn64.p, c.alphas.p, c.Xc.p, nb);
    }
    if (c.h.gam != 0) {
      const int gg = elem_grid((int64_t)(M - 1) * N);
      k_gamma_part<<<dim3(gg, nb), 256, 0, c.st>>>(c.Xc.p, MN, M, N, c.h.gam, c.part2.p);
      post_launch(c);
      reduce_to(c, c.part2.p, gg, c.lsout.p + kBatchLS, nb);
    }
    if (tc_screen) {
      // one tensor-core product over the probes' columns (split-BF16x3,
      // FP32 accumulation: F.dX to ~2^-16 of itself)
      tc_probe_products(c, c.Xc.p, c.x0c.p, nb);
      k_dres_part<<<dim3(g2, nb), 256, 0, c.st>>>(c.fdx32.p, c.r0_32.p, c.flo.p, D, N, (int64_t)nb * N, N, c.part.p);
    } else {
      k_delta32<<<dim3(g, nb), 256, 0, c.st>>>(c.Xc.p, c.x0c.p, MN, c.d32.p);
      post_launch(c);
      launch_band_gemm32(c, heuristic_tile(D, N, nb), c.flo.p, c.fw.p, c.foff.p, c.fval32.p, c.d32.p, D, N, 1.0f,
                         c.fdx32.p, nullptr, nb, MN, DN);
      k_dres_part<<<dim3(g2, nb), 256, 0, c.st>>>(c.fdx32.p, c.r0_32.p, c.flo.p, D, N, N, DN, c.part.p);
    }
    post_launch(c);
    reduce_to(c, c.part.p, g2, c.lsout.p + 3 * kBatchLS, nb);
    CK(cudaMemcpyAsync(c.pin, c.lsout.p, 4 * kBatchLS * sizeof(double), cudaMemcpyDeviceToHost, c.st));
    CK(cudaStreamSynchronize(c.st));
    for (int k = 0; k < nb; ++k) {
      xmin[k] = stage2 ? c.pin[2 * kBatchLS + k] : 0.0;
      dL[k] = c.pin[3 * kBatchLS + k] + (c.h.gam != 0 ? c.pin[kBatchLS + k] - Lgam0 : 0.0);
    }
    c.n_lsL += nb;
  };
  // the slope probe alpha = dx (404, 450) as an objective change (a
  // difference of two FP64 objectives ~1e-9 apart is what the reference
  // divides by dx; here it is computed directly), screened together with
  // the first two steps 1 and 0.75 (the full step is usually taken)
  double qa[kBatchLS], xmin[kBatchLS], dl[kBatchLS];
  qa[0] = 0.0 + kDx;
  qa[1] = 1.0;
  qa[2] = 1.0 * 0.75;
  screen(qa, 3, dl, xmin);
  LSState ls;
  ls.L0 = L0;
  ls.df = dl[0] / kDx;
  dlalpha = ls.df;
  bool screened_stop = false;
  double stop_a = 0.0;  // alpha of the probe where the screened sequence stopped
  ls.next_a = qa[2] * 0.75;
  for (int k = 1; k < 3 && !ls.done; ++k)
    if (ls_take(c, ls, stage2, qa[k], ls.L0 + dl[k], xmin[k])) {
      screened_stop = true;
      stop_a = qa[k];
    }
  while (!ls.done && ls.i <= kMaxLS) {
    const int nb = std::min(kBatchLS, kMaxLS - ls.i + 1);
    for (int k = 0; k < nb; ++k) {
      qa[k] = ls.next_a;
      ls.next_a = ls.next_a * 0.75;
    }
    screen(qa, nb, dl, xmin);
    for (int k = 0; k < nb && !ls.done; ++k)
      if (ls_take(c, ls, stage2, qa[k], ls.L0 + dl[k], xmin[k])) {
        screened_stop = true;
        stop_a = qa[k];
      }
  }
  // FP64 objective and sufficient-decrease check of the chosen step
  if (ls.alphamin != 0.0) {
    double a1[1] = {ls.alphamin}, Lv[1], xv[1];
    eval_candidates(c, a1, 1, stage2, Lv, xv);
    const double armijo = std::fma(0.1 * ls.alphamin, ls.df, ls.L0);
    const bool ok = Lv[0] <= armijo && (!stage2 || xv[0] >= -kFeasTol);
    if (!ok && screened_stop && ls.i <= kMaxLS) {
      // continue the reference's sequence in FP64 after the screened stop
      LSState f = ls;
      f.done = false;
      f.next_a = stop_a * 0.75;  // the probe after the screened stop
      f.lm = (!stage2 || xv[0] >= -kFeasTol) ? Lv[0] : kHuge;
      f.alphamin = (f.lm < kHuge) ? ls.alphamin : 0.0;
      ls_continue_fp64(c, f, stage2, 2);
      ls = f;
    } else if (!ok && !(Lv[0] < ls.L0)) {
      ls.alphamin = 0.0;  // no FP64 decrease: keep X (the reference's alpha = 0 case)
    }
  }
  alpha = ls.alphamin;
}

// conv_test (1034-1067) on the context's X; leaves the full space selected.
// with_extra: sc[SC_TMP + 1] (written by the caller's earlier kernels) is
// read back in the same transfer into c.pin[1].
static double op_conv(Ctx& c, bool tprint, bool with_extra = false) {
  Scope s(c.timers, "conv_test");
  const int M = (int)c.h.M, N = (int)c.h.N;
  if (!c.fullspace) rebuild_x(c);
  c.fullspace = true;
  op_dL(c);
  DBuf<double> lam;
  if (tprint && c.verbose) lam.alloc(M);
  k_conv_rows_t<<<cdiv(M, 32), kTileThreads, 0, c.st>>>(c.X.p, c.G.p, M, N, c.part.p,
                                                        (tprint && c.verbose) ? lam.p : nullptr);
  post_launch(c);
  if (c.exact) {
    k_seqsum<<<1, 32, 0, c.st>>>(c.part.p, M, nullptr, c.sc.p + SC_TMP, 1, nullptr);
    post_launch(c);
  } else {
    reduce_to(c, c.part.p, M, c.sc.p + SC_TMP);
  }
  read_back(c, c.sc.p + SC_TMP, with_extra ? 2 : 1);
  const double conv = std::sqrt(c.pin[0] / ((double)N * (double)M));
  if (tprint && c.verbose) {
    std::vector<double> hl(M), hg((size_t)M * N);
    CK(cudaMemcpyAsync(hl.data(), lam.p, M * 8, cudaMemcpyDeviceToHost, c.st));
    CK(cudaMemcpyAsync(hg.data(), c.G.p, (size_t)M * N * 8, cudaMemcpyDeviceToHost, c.st));
    CK(cudaStreamSynchronize(c.st));
    for (int i = 0; i < M; ++i) {
      double m2 = kHuge;
      for (int n = 0; n < N; ++n) m2 = std::min(m2, hg[(size_t)i * N + n] + hl[i]);
      ListLine l;
      l.s("lambda").i8(i + 1).r8(hl[i]).r8(m2).print();
    }
  }
  return conv;
}

static void set_full_space(Ctx& c) {
  c.fullspace = true;
  CK(cudaMemsetAsync(c.maxr.p, 0xff, c.h.M * sizeof(int32_t), c.st));  // maxr = -1
}

struct SolveState {
  double L0 = 0, norm_der = 0, conv = 0, alpha = 0, xmin = 0, dlalpha = 0;
  int64_t outer = 0;
  double t0 = 0;
};

static double wall() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Mode 2 (1953-2136), before the CG: the stage's space (stage 2: the max
// column placeholder, 1970-1983) and the gradient.  Returns bdfac, the
// preconditioner's factor of the space.
static double outer_pre_cg(Ctx& c, int oiter) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  c.fullspace = (oiter == 1);
  if (!c.fullspace) {
    k_stage2_start_t<<<cdiv(M, 32), kTileThreads, 0, c.st>>>(c.X.p, c.maxr.p, M, N, 1);
    post_launch(c);
    if (c.exact) {
      touch_x(c);
    } else {
      // mixed path: the placeholder is replaced by the next rebuild, which
      // restores X to within ulps; only the reduced gradient (new maxr)
      // must be derived again
      c.G_ver = -1;
    }
  } else {
    set_full_space(c);
  }
  op_dL(c);
  if (c.precision == PQDTS_MIXED && c.refine_option == 1 && !c.fullspace) c.refine = true;
  return c.fullspace ? 1.0 : 2.0;
}

// Whether this iteration's CG runs in FP32 (the mixed solver before its
// final refinement).
static bool cg_in_fp32(const Ctx& c) { return c.precision == PQDTS_MIXED && !c.refine; }

// Mode 2 after the CG: the two-metric direction (2092-2104) and the line
// search; the mixed solver switches to its FP64 refinement once an FP32
// Newton direction stops giving progress in stage 2.
static void outer_post_cg(Ctx& c, SolveState& st, double bdfac, bool fp32) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  const int g = elem_grid((int64_t)M * N);
  if (c.precision == PQDTS_MIXED && c.refine) c.n_refine++;
  op_dL(c);
  const int32_t* mr = c.fullspace ? nullptr : c.maxr.p;
  if (fp32) k_twometric32<<<g, 256, 0, c.st>>>(c.cg32.sn.p, c.G.p, c.ik.p, mr, c.bdiag.p, bdfac, M, N, c.sn64.p);
  else k_twometric<double><<<g, 256, 0, c.st>>>(c.cg64.sn.p, c.G.p, c.ik.p, mr, c.bdiag.p, bdfac, M, N, c.sn64.p);
  post_launch(c);
  if (c.exact) line_search(c, !c.fullspace, st.alpha, st.dlalpha);
  else line_search_mixed(c, !c.fullspace, st.alpha, st.dlalpha);
  if (c.precision == PQDTS_MIXED && !c.refine && !c.fullspace && (st.alpha == 0.0 || st.dlalpha >= 0.0))
    c.refine = true;
}

static void outer_tail(Ctx& c, SolveState& st);

// One outer iteration of mode 2 (1953-2136) or mode 1 (1934-1951, 2111-2136).
static void outer_iteration(Ctx& c, int mode, int oiter, SolveState& st) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  const int64_t MN = (int64_t)M * N;
  const int g = elem_grid(MN);
  if (mode == 1) {
    c.fullspace = false;
    k_stage2_start_t<<<cdiv(M, 32), kTileThreads, 0, c.st>>>(c.X.p, c.maxr.p, M, N, 0);
    post_launch(c);
    touch_x(c);
    op_dL(c);
    k_neg_copy<<<g, 256, 0, c.st>>>(MN, c.G.p, c.sn64.p);
    post_launch(c);
    line_search(c, true, st.alpha, st.dlalpha);
  } else {
    const double bdfac = outer_pre_cg(c, oiter);
    const bool fp32 = cg_in_fp32(c);
    if (fp32) cg_solve32(c, bdfac);
    else cg_solve<double>(c, c.cg64, c.fval.p, c.tval.p, bdfac, nullptr);
    outer_post_cg(c, st, bdfac, fp32);
  }
  outer_tail(c, st);
}

// The end of an outer iteration (2111-2136): the update X + alpha s and its
// projection (or, mixed path, the adopted line-search candidate), then L,
// dL, |der| and conv_test.
static void outer_tail(Ctx& c, SolveState& st) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  const int64_t MN = (int64_t)M * N;
  const int g = elem_grid(MN);
  // Mixed path: the chosen step was evaluated to FP64 accuracy as a
  // line-search candidate (projected, rebuilt, its residual and objective known): adopt
  // it instead of recomputing the same projection and banded product.
  int adopt = -1;
  if (!c.exact && st.alpha != 0.0 && c.cand_xver == c.xver && c.cand_stage2 == !c.fullspace)
    for (int b = 0; b < c.cand_B; ++b)
      if (c.cand_alpha[b] == st.alpha) {
        adopt = b;
        break;
      }
  st.xmin = 0.0;
  if (adopt >= 0) {
    const int64_t DN = c.h.D * c.h.N;
    CK(cudaMemcpyAsync(c.X.p, c.Xc.p + (size_t)adopt * MN, MN * sizeof(double), cudaMemcpyDeviceToDevice, c.st));
    touch_x(c);
    k_scale_copy<<<elem_grid(DN), 256, 0, c.st>>>(DN, 2.0, c.Rst.p + (size_t)adopt * DN, c.R.p);
    post_launch(c);
    c.R_ver = c.xver;
    c.L_cache = c.cand_L[adopt];
    c.Lgam_cache = c.cand_Lgam[adopt];
    c.L_ver = c.xver;
    if (!c.fullspace) {
      c.rebuilt_ver = c.xver;
      st.xmin = c.cand_xmin[adopt];
    }
  } else if (st.alpha != 0.0) {
    k_axpy<<<g, 256, 0, c.st>>>(MN, st.alpha, c.sn64.p, c.X.p);
    post_launch(c);
    touch_x(c);
  }
  if (adopt >= 0) {
  } else if (c.fullspace) {
    Scope s(c.timers, "doproj");
    project_rows(c, c.X.p, nullptr, nullptr, c.X.p, 1);
    touch_x(c);
  } else {
    Scope s(c.timers, "doproj2");
    const int gb = cdiv(M, 32);  // 32-row tiles
    k_cand_proj2_t<<<dim3(gb, 1), kTileThreads, 0, c.st>>>(c.X.p, nullptr, nullptr, c.X.p, MN, c.maxr.p, M, N, 0,
                                                         c.part2.p);
    post_launch(c);
    touch_x(c);
    c.rebuilt_ver = c.xver;  // doproj2 ends with the max-column rebuild
    reduce_to(c, c.part2.p, gb, c.sc.p + SC_TMP, 1, true, 0.0);
    read_back(c, c.sc.p + SC_TMP, 1);
    st.xmin = c.pin[0];
  }
  st.L0 = op_L(c);
  op_dL(c);
  // |der|^2 of this space's gradient, read back with conv_test's value
  dot_dev(c, c.G.p, c.G.p, c.sc.p + SC_TMP + 1);
  st.conv = op_conv(c, false, true);
  st.norm_der = c.pin[1];
  st.outer++;
}

static void print_iter(Ctx& c, int oiter, int iiter, int mode, const SolveState& st, double t1) {
  if (!c.verbose) return;
  const double t2 = wall();
  ListLine l;
  l.s("iter").i4(oiter).i4(iiter).s("L=").r8(st.L0).s("max(abs(c))").r8(st.xmin).s("conv").r8(st.conv);
  l.s("||der||=").r8(std::sqrt(st.norm_der)).s("mode=").i4(mode).s("alpha=").r8(st.alpha).s("dlalpha=").r8(st.dlalpha);
  l.s("dt=").r8(t2 - t1).s("ttot=").r8(t2 - st.t0).print();
  fflush(stdout);
}

static void run_stage(Ctx& c, int mode, int oiter, int maxiiter, double conv_thres, int output, SolveState& st) {
  st.dlalpha = -kHuge;
  for (int iiter = 1; iiter <= maxiiter; ++iiter) {
    const double t1 = wall();
    if (mode == 2 && oiter == 1 && (std::fabs(st.dlalpha) < kStage1Exit || st.dlalpha > 0)) {
      if (c.verbose) {
        ListLine l;
        l.s("stopping inner iteration because dldlpha is small").r8(st.dlalpha).print();
      }
      break;
    }
    outer_iteration(c, mode, oiter, st);
    print_iter(c, oiter, iiter, mode, st, t1);
    if (st.conv < conv_thres) break;
    if (c.target_L > 0 && st.L0 <= c.target_L) {
      c.target_hit = true;
      break;
    }
  }
  st.conv = op_conv(c, output >= 3);
  c.timers.flush();
}

static void get_x_colmajor(Ctx& c, double* out) {
  const int64_t M = c.h.M, N = c.h.N;
  std::vector<double> rm((size_t)M * N);
  CK(cudaMemcpyAsync(rm.data(), c.X.p, rm.size() * 8, cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  c.d2h += (int64_t)rm.size() * 8;
  for (int64_t i = 0; i < M; ++i)
    for (int64_t n = 0; n < N; ++n) out[i + n * M] = rm[(size_t)i * N + n];
}

static void set_x_colmajor(Ctx& c, const double* in) {
  const int64_t M = c.h.M, N = c.h.N;
  std::vector<double> rm((size_t)M * N);
  for (int64_t i = 0; i < M; ++i)
    for (int64_t n = 0; n < N; ++n) rm[(size_t)i * N + n] = in[i + n * M];
  CK(cudaMemcpyAsync(c.X.p, rm.data(), rm.size() * 8, cudaMemcpyHostToDevice, c.st));
  CK(cudaStreamSynchronize(c.st));
  c.h2d += (int64_t)rm.size() * 8;
  touch_x(c);
}

static void download_rowmajor_to_col(Ctx& c, const double* dev, double* out) {
  const int64_t M = c.h.M, N = c.h.N;
  std::vector<double> rm((size_t)M * N);
  CK(cudaMemcpyAsync(rm.data(), dev, rm.size() * 8, cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  for (int64_t i = 0; i < M; ++i)
    for (int64_t n = 0; n < N; ++n) out[i + n * M] = rm[(size_t)i * N + n];
}

static void fill_stats(Ctx& c, const SolveState& st, double secs, double* stats) {
  if (!stats) return;
  stats[0] = st.L0;
  stats[1] = st.conv;
  stats[2] = std::sqrt(st.norm_der);
  stats[3] = (double)st.outer;
  stats[4] = (double)c.n_cg;
  stats[5] = (double)c.n_lsL;
  stats[6] = (double)c.n_refine;
  stats[7] = secs;
}

// Mixed path, end of a stage: Pi >= 0 exactly.  Rows with a negative entry
// are projected onto the simplex in place (a change of ~1e-12 at most, the
// size of the reference's own tolerance, pqdts.f90:424); when any row moved,
// the reported objective is that of the projected X (conv stays the stage's
// last conv_test).  The FP64 drop-in keeps the reference's -1e-12 allowance
// and its bit-exact iterate.
static void nonneg_x(Ctx& c, SolveState& st) {
  const int M = (int)c.h.M, N = (int)c.h.N;
  CK(cudaMemsetAsync(c.icount.p, 0, sizeof(long long), c.st));
  k_nonneg_rows<<<cdiv((int64_t)M * 32, 256), 256, 0, c.st>>>(c.X.p, M, N, (unsigned long long*)c.icount.p);
  post_launch(c);
  long long moved = 0;
  CK(cudaMemcpyAsync(&moved, c.icount.p, sizeof(long long), cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  if (moved == 0) return;
  touch_x(c);
  c.fullspace = true;
  st.L0 = op_L(c);
}

// The start of a solve (1908-1915): counters, the seeded first maxr, the
// objective and gradient of the starting point (full space) and |der|^2.
static void solve_prologue(Ctx& c, SolveState& st) {
  c.n_cg = c.n_lsL = c.n_refine = 0;
  c.refine = false;
  CK(cudaMemcpyAsync(c.maxr.p, c.h_maxr.data(), c.h.M * 4, cudaMemcpyHostToDevice, c.st));
  c.h2d += c.h.M * 4;
  touch_x(c);
  c.fullspace = true;
  st.L0 = op_L(c);
  op_dL(c);
  dot_dev(c, c.G.p, c.G.p, c.sc.p + SC_TMP);
  read_back(c, c.sc.p + SC_TMP, 1);
  st.norm_der = c.pin[0];
}

static void solve(Ctx& c, int mode, int maxiiter, double conv_thres, int start_stage, int output, pqdts_stage_cb cb,
                  void* user, double* stats) {
  need_problem(c);
  if (mode != 1 && mode != 2) throw Err(PQDTS_E_ARG, "mode must be 1 or 2");
  if (start_stage < 1 || start_stage > 2) throw Err(PQDTS_E_ARG, "start_stage must be 1 or 2");
  SolveState st;
  solve_prologue(c, st);
  if (c.verbose) {
    ListLine l;
    l.s("iter").i4(0).i4(0).s("L=").r8(st.L0).s("||der||=").r8(std::sqrt(st.norm_der)).s("dt=").r8(0.0).s("ttot=").r8(0.0);
    l.print();
  }
  const double t0 = wall();
  st.t0 = t0;
  const int tmin = c.timers.begin("min");
  c.target_hit = false;
  for (int oiter = start_stage; oiter <= 2 && !c.target_hit; ++oiter) {
    run_stage(c, mode, oiter, maxiiter, conv_thres, output, st);
    if (c.precision == PQDTS_MIXED) nonneg_x(c, st);
    if (cb) {
      std::vector<double> xh((size_t)c.h.M * c.h.N);
      get_x_colmajor(c, xh.data());
      cb(user, oiter, xh.data());
    }
  }
  c.timers.end(tmin);
  c.timers.flush();
  CK(cudaStreamSynchronize(c.st));
  fill_stats(c, st, wall() - t0, stats);
}

// ---------------------------------------------------------------------------
// Lockstep solve of a group of mixed-precision instances that share F (the
// resampled / gamma-swept members of a batch).  Each member is a context of
// its own (its P, gamma, iterate, line search, stages), all on the group
// context's stream; in every round each member runs up to its CG (stage
// logic and gradient), the members whose CG is in FP32 then run it jointly
// -- one launch per CG phase for all of them, the tensor-core products over
// the group context's widened problem (M, G*N, D: the members' V side by
// side; batch_cg.cuh) -- and each member finishes its outer iteration (line
// search, update, conv_test).  A member's arithmetic is the single-instance
// solver's; its stage and stopping logic is run_stage / solve's, as a state
// machine (mode 2, no stage callback, no printing).
// ---------------------------------------------------------------------------
struct MemberRun {
  Ctx* c = nullptr;
  SolveState st;
  int oiter = 1, iiter = 0;
  bool in_stage = false, finished = false, stepped = false, fp32 = false;
  double bdfac = 1.0, t0 = 0.0;
  int maxiiter = 0;
  double conv_thres = 0.0;
  double* stats = nullptr;
};

static void member_end_stage(MemberRun& m) {
  Ctx& c = *m.c;
  m.st.conv = op_conv(c, false);
  c.timers.flush();
  if (c.precision == PQDTS_MIXED) nonneg_x(c, m.st);
  m.in_stage = false;
  m.oiter++;
}

// Runs the member up to its next CG (run_stage's loop head and the outer
// iteration's first part); false once its solve has finished.
static bool member_next(MemberRun& m) {
  Ctx& c = *m.c;
  for (;;) {
    if (m.finished) return false;
    if (!m.in_stage) {
      if (m.oiter > 2 || c.target_hit) {
        CK(cudaStreamSynchronize(c.st));
        fill_stats(c, m.st, wall() - m.t0, m.stats);
        m.finished = true;
        return false;
      }
      m.st.dlalpha = -kHuge;
      m.iiter = 0;
      m.in_stage = true;
    }
    const bool stage1_exit = m.oiter == 1 && (std::fabs(m.st.dlalpha) < kStage1Exit || m.st.dlalpha > 0);
    if (m.iiter >= m.maxiiter || stage1_exit) {
      member_end_stage(m);
      continue;
    }
    m.iiter++;
    m.bdfac = outer_pre_cg(c, m.oiter);
    m.fp32 = cg_in_fp32(c);
    return true;
  }
}

// The rest of the member's outer iteration and run_stage's exit tests.
static void member_after_cg(MemberRun& m) {
  Ctx& c = *m.c;
  outer_post_cg(c, m.st, m.bdfac, m.fp32);
  outer_tail(c, m.st);
  if (m.st.conv < m.conv_thres) {
    member_end_stage(m);
  } else if (c.target_L > 0 && m.st.L0 <= c.target_L) {
    c.target_hit = true;
    member_end_stage(m);
  }
}

// The FP32 CG of the members listed in `in_cg` (their cg32_begin queued),
// one launch per phase for all of them on g's stream.
static void group_cg32(Ctx& g, std::vector<MemberRun>& ms, const std::vector<int>& in_cg) {
  const int G = (int)ms.size();
  const int M = (int)g.h.M, N = (int)ms[0].c->h.N;
  const int64_t Nw = g.h.N;  // G * N
  g.h_memtab.assign(G, CGMember{});
  for (int j : in_cg) {
    Ctx& c = *ms[j].c;
    CGMember& e = g.h_memtab[j];
    e.p = c.cg32.p.p;
    e.z = c.cg32.z.p;
    e.rs = c.cg32.rs.p;
    e.Hp = c.cg32.Hp.p;
    e.sn = c.cg32.sn.p;
    e.r = c.cg32.r.p;
    e.rsq = c.rsq32.p;
    e.maxr = c.fullspace ? nullptr : c.maxr.p;
    e.ik = c.ik.p;
    e.sc = c.sc.p;
    e.part_rz = c.part.p;
    e.part_rr = c.part2.p;
    e.dpart = c.part.p;
    e.cnt_epi = c.counters.p + 4;
    e.cnt_step = c.counters.p + 1;
    e.log = c.cglog.p;
    e.c2gam = (float)(2.0 * c.h.gam);
    e.active = 1;
  }
  g.memtab.alloc(G);
  CK(cudaMemcpyAsync(g.memtab.p, g.h_memtab.data(), G * sizeof(CGMember), cudaMemcpyHostToDevice, g.st));
  CK(cudaMemsetAsync(g.counters.p + 6, 0, sizeof(unsigned), g.st));
  CK(cudaMemsetAsync(g.sc.p + SC_DONE, 0, sizeof(double), g.st));
  const int active = (int)in_cg.size();
  const CGGroup grp{g.counters.p + 6, g.sc.p, active};
  const int RB = epi_rows(g, M);
  const int gs = std::min(elem_grid((int64_t)M * N), cdiv(M, 8));
  auto iteration = [&](bool first) {
    k_cg_lift_split_b<32><<<dim3(cdiv(M, 32), G), dim3(32, 32), 0, g.st>>>(g.memtab.p, first ? 0 : 1, M, N, g.tc_mp,
                                                                           g.vt_hi.p, g.vt_lo.p);
    post_launch(g);
    tc_forward(g, g.sched.tc_splits1, g.sched.tc_persistent, g.sc.p);
    tc_product(g, g.tcFt, g.map_yt_hi, g.map_yt_lo, M, g.sched.tc_splits, 0, 1.0f, g.hpart32.p, nullptr, nullptr, 0,
               g.sc.p, g.sched.tc_persistent);
    k_hvp_epi32_rows_b<<<dim3(cdiv(M, RB), G), kEpiThreads, 0, g.st>>>(g.memtab.p, g.hpart32.p, Nw,
                                                                        (int64_t)M * Nw, M, N, RB,
                                                                        g.sched.tc_splits);
    post_launch(g);
    k_cg_step32_b<<<dim3(gs, G), 256, 0, g.st>>>(g.memtab.p, grp, M, N, kMaxCG);
    post_launch(g);
  };
  cg_chunks(g, {100, (uint64_t)active, 0, 0}, iteration);
  for (int j : in_cg) {
    Ctx& c = *ms[j].c;
    read_back(c, c.sc.p, SC_NSC);
    cg32_end(c, (int)c.pin[SC_ITER]);
  }
}

// Whether a group of instances of this shape can take the joint CG:
// tensor-core products on the group context and the multi-row epilogue.
static bool group_ready(const Ctx& g, int64_t N) {
  (void)N;
  return g.have_problem && g.precision == PQDTS_MIXED && g.sched.tc && g.tc_ready && g.rows_option != 0;
}

static void group_solve(Ctx& g, std::vector<MemberRun>& ms) {
  for (MemberRun& m : ms) {
    Ctx& c = *m.c;
    need_problem(c);
    solve_prologue(c, m.st);
    m.t0 = wall();
    m.st.t0 = m.t0;
    c.target_hit = false;
  }
  std::vector<int> in_cg;
  for (;;) {
    in_cg.clear();
    bool any = false;
    for (int j = 0; j < (int)ms.size(); ++j) {
      MemberRun& m = ms[j];
      m.stepped = member_next(m);
      if (!m.stepped) continue;
      any = true;
      if (m.fp32) {
        cg32_begin(*m.c, m.bdfac);
        in_cg.push_back(j);
      } else {  // the member's FP64 refinement CG, on its own
        cg_solve<double>(*m.c, m.c->cg64, m.c->fval.p, m.c->tval.p, m.bdfac, nullptr);
      }
    }
    if (!any) break;
    if (!in_cg.empty()) group_cg32(g, ms, in_cg);
    for (MemberRun& m : ms)
      if (m.stepped) member_after_cg(m);
  }
}

// ---------------------------------------------------------------------------
// Autotuner: the banded products' launch schedule (FP32 tile shapes and K
// splits, FP64 transposed-product block shape) timed on this problem's F at
// set-up and remembered for the process per size bucket (device, precision,
// N, and the log2 buckets of M, D and the mean band width), so instances of
// one bucket (a resampled or gamma-swept batch) are tuned once.
// ---------------------------------------------------------------------------
static std::mutex g_sched_mu;
static std::map<std::array<int64_t, 10>, Schedule> g_sched;

static int ilog2_ceil(int64_t v) {
  int k = 0;
  while (((int64_t)1 << k) < v) ++k;
  return k;
}

struct EventPair {
  cudaEvent_t a = nullptr, b = nullptr;
  EventPair() {
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
  }
  ~EventPair() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

// Mean device time of one call of fn (ms): one untimed call, then `reps`.
template <class F>
static float time_calls(Ctx& c, int reps, F&& fn) {
  fn();
  EventPair ev;
  CK(cudaEventRecord(ev.a, c.st));
  for (int r = 0; r < reps; ++r) fn();
  CK(cudaEventRecord(ev.b, c.st));
  CK(cudaEventSynchronize(ev.b));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, ev.a, ev.b));
  return ms / (float)reps;
}

// A schedule is only timed when one launch of the heuristic is shorter than
// this (large problems fill the GPU with the heuristic's shapes anyway).
constexpr float kTuneMaxMs = 20.0f;
constexpr int kTuneReps = 3;

static Schedule heuristic_schedule(const HostProblem& h) {
  Schedule s;
  const int M = (int)h.M, N = (int)h.N, D = (int)h.D;
  s.fwd_tile = heuristic_tile(D, N);
  s.trn_tile = 0;
  const int64_t ctas = tile_ctas(0, M, N);
  s.trn_splits = (int)std::min<int64_t>(8, std::max<int64_t>(1, (2 * 152 + ctas - 1) / ctas));
  const TransShape sh = trans_shape(N);
  s.trans_threads = sh.threads;
  s.trans_cols = sh.C;
  return s;
}

// The Hessian row epilogue over `parts` partials (full space, no mask), as
// the CG runs it after the transposed product: part of that product's cost.
static void tune_epilogue(Ctx& c, int parts) {
  hvp_epilogue(c, c.cg32.p.p, nullptr, nullptr, c.cg32.Hp.p, c.part.p, nullptr, parts);
}

static void tune_schedule(Ctx& c, Schedule& s) {
  const int M = (int)c.h.M, N = (int)c.h.N, D = (int)c.h.D;
  const int64_t MN = (int64_t)M * N;
  // FP64 transposed product: for each column count C, the thread count with
  // the fewest passes over the CSR row, then the fewest idle lanes (not for
  // a mixed problem whose gradient and checks run in double-FP32: there the
  // FP64 products serve only the final refinement, on heuristic shapes)
  if (c.precision != PQDTS_MIXED || !(c.df_fwd && c.df_trans)) {
    CGBufs<double>& b = c.cg64;
    CK(cudaMemsetAsync(b.R2.p, 0, b.R2.n * sizeof(double), c.st));
    CK(cudaMemsetAsync(b.p.p, 0, b.p.n * sizeof(double), c.st));
    auto run = [&](TransShape sh) {
      launch_trans_shape<double, true>(c, sh, c.tval.p, b.R2.p, b.p.p, nullptr, 0, 2.0 * c.h.gam, nullptr, b.Hp.p,
                                       nullptr, nullptr, nullptr);
    };
    const TransShape h0{s.trans_threads, s.trans_cols};
    float best = time_calls(c, kTuneReps, [&] { run(h0); });
    if (best < kTuneMaxMs) {
      for (int C : {1, 2, 4, 8}) {
        TransShape cand{0, C};
        int64_t bp = INT64_MAX, bw = INT64_MAX;
        for (int t = 32; t <= 256; t += 32) {
          const int64_t per = (int64_t)t * C, passes = (N + per - 1) / per, waste = passes * per - N;
          if (passes < bp || (passes == bp && waste < bw)) {
            bp = passes;
            bw = waste;
            cand.threads = t;
          }
        }
        if (cand.threads == h0.threads && cand.C == h0.C) continue;
        const float t = time_calls(c, kTuneReps, [&] { run(cand); });
        if (t < best) {
          best = t;
          s.trans_threads = cand.threads;
          s.trans_cols = cand.C;
        }
      }
    }
    // the row-flattened forms (same bits), where they apply
    if (c.rows_option != 0 && rows_per_block(N) > 0) {
      if (c.t_contiguous) {
        TransShape rw{s.trans_threads, s.trans_cols};
        rw.rows = 1;
        const float t = time_calls(c, kTuneReps, [&] { run(rw); });
        s.trans_rows = (c.rows_option == 1 || t < best) ? 1 : 0;
      }
      auto fwd64 = [&](int rows) {
        launch_fwd<double, 1>(c, c.fval.p, b.p.p, 0, nullptr, b.R2.p, 1, nullptr, rows);
      };
      const float t0 = time_calls(c, kTuneReps, [&] { fwd64(0); });
      const float t1 = t0 < kTuneMaxMs ? time_calls(c, kTuneReps, [&] { fwd64(1); }) : t0;
      s.fwd_rows = (c.rows_option == 1 || t1 < t0) ? 1 : 0;
    }
  }
  if (c.precision != PQDTS_MIXED) return;
  if (s.tc) {
    // tensor-core products: N tile width x K splits of the F^T product
    // (partials of at most 1 GiB)
    const int max_splits = (int)std::max<int64_t>(1, std::min<int64_t>(8, ((int64_t)1 << 30) / (MN * 4)));
    c.hpart32.alloc((size_t)std::max(max_splits, s.tc_splits) * MN);
    CK(cudaMemsetAsync(c.vt_hi.p, 0, c.vt_hi.n * sizeof(__nv_bfloat16), c.st));
    CK(cudaMemsetAsync(c.vt_lo.p, 0, c.vt_lo.n * sizeof(__nv_bfloat16), c.st));
    CK(cudaMemsetAsync(c.yt_hi.p, 0, c.yt_hi.n * sizeof(__nv_bfloat16), c.st));
    CK(cudaMemsetAsync(c.yt_lo.p, 0, c.yt_lo.n * sizeof(__nv_bfloat16), c.st));
    int pers = 0, sp1 = 1;
    const int64_t DN = (int64_t)D * N;
    const int max_splits1 = (int)std::max<int64_t>(1, std::min<int64_t>(4, ((int64_t)1 << 30) / (DN * 4)));
    if (max_splits1 > 1) c.ypart.alloc((size_t)max_splits1 * DN);
    auto fwd = [&] { tc_forward(c, sp1, pers, nullptr); };
    auto trn = [&](int sp) {  // the F^T product and the epilogue that sums its sp partials
      tc_product(c, c.tcFt, c.map_yt_hi, c.map_yt_lo, M, sp, 0, 1.0f, c.hpart32.p, nullptr, nullptr, 0, nullptr,
                 pers);
      tune_epilogue(c, sp);
    };
    float best = 0.0f;
    int best_bn = s.tc_bn, best_sp = s.tc_splits, best_pers = s.tc_persistent, best_sp1 = 1;
    bool first = true, large = false;
    for (int mult : {1, 2, 4}) {
      const int bn = tc_tile_n(N, mult);
      if (!first && (bn == c.tc_bn || bn < 32)) continue;
      tc_configure(c, bn);
      for (int pv : {0, 1}) {
        if (c.tc_persistent_option >= 0 && pv != c.tc_persistent_option) continue;
        pers = pv;
        // the F.V product: K splits only help when its tiles do not fill the GPU
        int sp1_best = 1;
        sp1 = 1;
        float t1 = time_calls(c, kTuneReps, fwd);
        const int64_t fwd_tiles = (int64_t)cdiv(N, bn) * c.tcF.blocks;
        if (t1 < kTuneMaxMs && fwd_tiles < c.num_sms)
          for (int cand : {2, 4}) {
            if (cand > max_splits1) continue;
            sp1 = cand;
            const float t = time_calls(c, kTuneReps, fwd);
            if (t < t1 * 0.97f) {
              t1 = t;
              sp1_best = cand;
            }
          }
        sp1 = sp1_best;
        int sp_best = s.tc_splits;
        float t2 = time_calls(c, kTuneReps, [&] { trn(sp_best); });
        if (t1 + t2 < kTuneMaxMs)
          for (int sp : {1, 2, 3, 4, 6, 8}) {
            if (sp > max_splits || sp == s.tc_splits) continue;
            const float t = time_calls(c, kTuneReps, [&] { trn(sp); });
            if (t < t2 * (sp > sp_best ? 0.97f : 1.0f)) {
              t2 = t;
              sp_best = sp;
            }
          }
        if (first || t1 + t2 < best) {
          best = t1 + t2;
          best_bn = bn;
          best_sp = sp_best;
          best_pers = pv;
          best_sp1 = sp1_best;
        }
        first = false;
        if (t1 + t2 >= kTuneMaxMs) large = true;
      }
      if (large) break;
    }
    s.tc_persistent = best_pers;
    s.tc_splits1 = best_sp1;
    tc_configure(c, best_bn);
    s.tc_bn = best_bn;
    s.tc_splits = best_sp;
    return;
  }
  CGBufs<float>& b = c.cg32;
  CK(cudaMemsetAsync(b.p.p, 0, b.p.n * sizeof(float), c.st));
  CK(cudaMemsetAsync(b.R2.p, 0, b.R2.n * sizeof(float), c.st));
  auto fwd = [&](int tile) {
    launch_band_gemm32(c, tile, c.flo.p, c.fw.p, c.foff.p, c.fval32.p, b.p.p, D, N, 2.0f, b.R2.p, nullptr);
  };
  float best = time_calls(c, kTuneReps, [&] { fwd(s.fwd_tile); });
  if (best < kTuneMaxMs)
    for (int tile = 0; tile < 3; ++tile) {
      if (tile == s.fwd_tile) continue;
      const float t = time_calls(c, kTuneReps, [&] { fwd(tile); });
      if (t < best) {
        best = t;
        s.fwd_tile = tile;
      }
    }
  // transposed product: tile x K splits, partials of at most 1 GiB
  const int max_splits = (int)std::max<int64_t>(1, std::min<int64_t>(8, ((int64_t)1 << 30) / (MN * 4)));
  c.hpart32.alloc((size_t)std::max(max_splits, s.trn_splits) * MN);
  auto trn = [&](int tile, int sp) {  // the F^T product and the epilogue that sums its sp partials
    launch_band_gemm32(c, tile, c.tlo.p, c.tw.p, c.toff.p, c.tbval32.p, b.R2.p, M, N, 1.0f, c.hpart32.p, nullptr,
                       sp, 0, MN, sp);
    tune_epilogue(c, sp);
  };
  best = time_calls(c, kTuneReps, [&] { trn(s.trn_tile, s.trn_splits); });
  if (best < kTuneMaxMs)
    for (int tile = 0; tile < 3; ++tile)
      for (int sp : {1, 2, 3, 4, 6, 8}) {
        if (sp > max_splits || (tile == s.trn_tile && sp == s.trn_splits)) continue;
        if (tile_ctas(tile, M, N) * sp > 16 * 152) continue;
        const float t = time_calls(c, kTuneReps, [&] { trn(tile, sp); });
        // more partials cost the epilogue a read each: require a clear gain
        if (t < best * (sp > s.trn_splits ? 0.97f : 1.0f)) {
          best = t;
          s.trn_tile = tile;
          s.trn_splits = sp;
        }
      }
}

static void choose_schedule(Ctx& c) {
  const HostProblem& h = c.h;
  setup_tc(c);
  Schedule s = heuristic_schedule(h);
  if (c.tc_ready) {
    s.tc = 1;
    s.tc_bn = c.tc_bn;
    s.tc_persistent = c.tc_persistent_option == 1 ? 1 : 0;
    const int64_t ctas = (int64_t)cdiv(h.N, c.tc_bn) * c.tcFt.blocks;
    s.tc_splits = (int)std::min<int64_t>(8, std::max<int64_t>(1, (152 + ctas - 1) / ctas));
  }
  if (c.autotune) {
    const int64_t wavg = h.D > 0 ? std::max<int64_t>(1, h.nnz() / h.D) : 1;
    const std::array<int64_t, 10> key{c.device,        c.precision,      h.N,
                                      ilog2_ceil(h.M),  ilog2_ceil(h.D),  ilog2_ceil(wavg),
                                      (int64_t)s.tc,    (int64_t)c.tc_persistent_option,
                                      (int64_t)c.rows_option, (int64_t)c.t_contiguous};
    std::lock_guard<std::mutex> lk(g_sched_mu);
    auto it = g_sched.find(key);
    if (it != g_sched.end()) {
      s = it->second;
      if (s.tc) tc_configure(c, s.tc_bn);
    } else {
      tune_schedule(c, s);
      s.tuned = 1;
      g_sched[key] = s;
    }
  }
  if (s.tc && c.tc_splits1_option > 0) s.tc_splits1 = c.tc_splits1_option;
  if (c.rows_option >= 0 && rows_per_block((int)h.N) > 0) {
    s.fwd_rows = c.rows_option;
    s.trans_rows = c.rows_option && c.t_contiguous ? 1 : 0;
  }
  c.sched = s;
  if (s.tc && s.tc_persistent) {  // tile lists of the persistent kernel, built before any capture
    tc_sched(c, c.tcF, c.tc_bn, std::max(1, s.tc_splits1));
    tc_sched(c, c.tcFt, c.tc_bn, s.tc_splits);
  }
  if (s.tc && s.tc_splits1 > 1) {
    const size_t need1 = (size_t)s.tc_splits1 * (size_t)h.D * (size_t)h.N;
    if (c.ypart.n != need1) c.ypart.alloc(need1);
  } else {
    c.ypart.release();
  }
  if (c.precision == PQDTS_MIXED) {
    const size_t need = (size_t)(s.tc ? s.tc_splits : s.trn_splits) * (size_t)h.M * (size_t)h.N;
    if (c.hpart32.n != need) c.hpart32.alloc(need);
  } else {
    c.hpart32.release();
  }
  read_back(c, c.sc.p, SC_NSC);
  check_tc_error(c);
}

// Internal F (pqdts.f90:1366-1466) computed on the device: each probe row's
// window (k_internal_windows, one thread per row scanning as the reference
// does) and its values (k_internal_values); the host then builds the
// transposed CSR and the Hessian diagonal from them as from any band input.
static void bands_internal_device(Ctx& c, HostProblem& h) {
  if (h.M != (h.D - 1) * (h.D - 1)) throw std::invalid_argument("M is not (D-1)**2");
  const int D = (int)h.D;
  const double sqrt_2pi = std::sqrt(2 * (4.0 * std::atan(1.0)));  // as the host fprob
  DBuf<int32_t> lo, w;
  DBuf<int64_t> off;
  DBuf<double> val;
  lo.alloc(D);
  w.alloc(D);
  k_internal_windows<<<cdiv(D, 128), 128, 0, c.st>>>(h.M, D, sqrt_2pi, lo.p, w.p);
  post_launch(c);
  h.flo.assign(D, -1);
  h.fw.assign(D, 0);
  CK(cudaMemcpyAsync(h.flo.data(), lo.p, (size_t)D * 4, cudaMemcpyDeviceToHost, c.st));
  CK(cudaMemcpyAsync(h.fw.data(), w.p, (size_t)D * 4, cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
  finish_offsets(h);
  if (h.fval.empty()) return;
  off.upload(h.foff.data(), D, c.st, nullptr);
  val.alloc(h.fval.size());
  k_internal_values<<<D, 256, 0, c.st>>>(D, sqrt_2pi, lo.p, w.p, off.p, val.p);
  post_launch(c);
  CK(cudaMemcpyAsync(h.fval.data(), val.p, h.fval.size() * 8, cudaMemcpyDeviceToHost, c.st));
  CK(cudaStreamSynchronize(c.st));
}

// Problem set-up shared by the entry points.
static void init_problem(Ctx& c, HostProblem&& h, int precision, SeededStream& rng) {
  if (precision != PQDTS_FP64 && precision != PQDTS_MIXED) throw Err(PQDTS_E_ARG, "precision must be 0 or 1");
  c.have_problem = false;
  c.h = std::move(h);
  finish_problem(c.h);
  c.h_maxr = initial_maxr(c.h.M, c.h.N, rng);
  c.precision = precision;
  setup_device(c);
  choose_schedule(c);
}

static void check_sizes(int64_t M, int64_t N, int64_t D) {
  if (M < 2 || N < 1 || D < 1) throw Err(PQDTS_E_ARG, "need M >= 2, N >= 1, D >= 1");
  if (M > INT32_MAX || N > INT32_MAX || D > INT32_MAX || M * N >= ((int64_t)1 << 31) || D * N >= ((int64_t)1 << 31))
    throw Err(PQDTS_E_ARG, "problem too large for 32-bit row indexing");
}

}  // namespace pqdts

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using pqdts::Ctx;
using pqdts::Err;

// Restores the thread's allocation stream on every exit path.
struct AllocStream {
  cudaStream_t saved;
  explicit AllocStream(cudaStream_t s) : saved(pqdts::t_alloc_stream) { pqdts::t_alloc_stream = s; }
  ~AllocStream() { pqdts::t_alloc_stream = saved; }
};

template <typename F>
static int guarded(Ctx* c, F&& f) {
  if (!c) return PQDTS_E_ARG;
  AllocStream as(c->st);
  try {
    if (c->st) {
      cudaError_t e = cudaSetDevice(c->device);
      if (e != cudaSuccess) throw Err(PQDTS_E_CUDA, cudaGetErrorString(e));
    }
    f();
    return PQDTS_OK;
  } catch (const Err& e) {
    c->err = e.what();
    return e.code;
  } catch (const std::invalid_argument& e) {
    c->err = e.what();
    return PQDTS_E_ARG;
  } catch (const std::bad_alloc&) {
    c->err = "host allocation failed";
    return PQDTS_E_NOMEM;
  } catch (const std::exception& e) {
    c->err = e.what();
    return PQDTS_E_CUDA;
  }
}

extern "C" {

// A context on `device`, with its own stream or (shared != null, the
// members of a batched group) on another context's stream.
static int create_ctx(int32_t device, cudaStream_t shared, pqdts_ctx** out) {
  if (!out) return PQDTS_E_ARG;
  *out = nullptr;
  Ctx* c = new (std::nothrow) Ctx();
  if (!c) return PQDTS_E_NOMEM;
  c->device = device;
  int rc = guarded(c, [&] {
    int n = 0;
    CK(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) throw Err(PQDTS_E_ARG, "no CUDA device " + std::to_string(device));
    CK(cudaSetDevice(device));
    if (shared) {
      c->st = shared;
      c->own_stream = false;
    } else {
      CK(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
    }
    CK(cudaMallocHost((void**)&c->pin, 64 * sizeof(double)));
    c->timers.st = c->st;
  });
  if (rc != PQDTS_OK) {
    fprintf(stderr, "pqdts_cuda_create: %s\n", c->err.c_str());
    if (c->st && c->own_stream) cudaStreamDestroy(c->st);
    delete c;
    return rc;
  }
  *out = c;
  return PQDTS_OK;
}

int pqdts_cuda_create(int32_t device, pqdts_ctx** out) { return create_ctx(device, nullptr, out); }

int pqdts_cuda_destroy(pqdts_ctx* c) {
  if (!c) return PQDTS_E_ARG;
  cudaSetDevice(c->device);
  if (c->st) cudaStreamSynchronize(c->st);
  if (c->pin) cudaFreeHost(c->pin);
  cudaStream_t st = c->own_stream ? c->st : nullptr;
  delete c;
  if (st) cudaStreamDestroy(st);
  return PQDTS_OK;
}

int pqdts_cuda_last_error(pqdts_ctx* c, char* buf, int64_t len) {
  if (!c || !buf || len <= 0) return PQDTS_E_ARG;
  snprintf(buf, (size_t)len, "%s", c->err.c_str());
  return PQDTS_OK;
}

int pqdts_cuda_kernel_launches(pqdts_ctx* c, int64_t* count) {
  if (!c || !count) return PQDTS_E_ARG;
  *count = c->launches.load();
  return PQDTS_OK;
}

int pqdts_cuda_set_verbose(pqdts_ctx* c, int32_t v) {
  if (!c) return PQDTS_E_ARG;
  c->verbose = v;
  return PQDTS_OK;
}

int pqdts_cuda_set_problem(pqdts_ctx* c, int64_t M, int64_t N, int64_t D, const int64_t* lo, const int64_t* hi,
                           const double* vals, const double* P, double gamma, int32_t precision) {
  return guarded(c, [&] {
    pqdts::check_sizes(M, N, D);
    if (!lo || !hi || !P) throw Err(PQDTS_E_ARG, "null band or P pointer");
    pqdts::HostProblem h;
    h.M = M;
    h.N = N;
    h.D = D;
    h.gam = gamma;
    int64_t tot = 0;
    for (int64_t d = 0; d < D; ++d)
      if (lo[d] >= 0) tot += hi[d] - lo[d] + 1;
    if (tot > 0 && !vals) throw Err(PQDTS_E_ARG, "null band values");
    pqdts::bands_from_bands(h, lo, hi, vals);
    h.P.assign(P, P + (size_t)D * N);
    pqdts::SeededStream rng;
    pqdts::init_problem(*c, std::move(h), precision, rng);
  });
}

int pqdts_cuda_set_problem_coo(pqdts_ctx* c, int64_t M, int64_t N, int64_t D, int64_t nnzF, const int32_t* Fr,
                               const int32_t* Fc, const double* Fv, int64_t nnzP, const int32_t* Pr, const int32_t* Pc,
                               const double* Pv, double gamma, int32_t precision) {
  return guarded(c, [&] {
    pqdts::check_sizes(M, N, D);
    pqdts::HostProblem h;
    h.M = M;
    h.N = N;
    h.D = D;
    h.gam = gamma;
    if (nnzF >= 0) {
      if (nnzF > 0 && (!Fr || !Fc || !Fv)) throw Err(PQDTS_E_ARG, "null F arrays");
      pqdts::bands_from_coo(h, nnzF, Fr, Fc, Fv);
    } else if (c->internal_f_option == 1 || (c->internal_f_option < 0 && precision == PQDTS_MIXED)) {
      pqdts::bands_internal_device(*c, h);
    } else {
      pqdts::bands_internal(h);
    }
    if (nnzP > 0 && (!Pr || !Pc || !Pv)) throw Err(PQDTS_E_ARG, "null P arrays");
    pqdts::SeededStream rng;
    pqdts::P_from_coo(h, nnzP, Pr, Pc, Pv, rng);
    pqdts::init_problem(*c, std::move(h), precision, rng);
  });
}

int pqdts_cuda_get_bands(pqdts_ctx* c, int64_t* lo, int64_t* hi, int64_t* nnz) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    for (int64_t d = 0; d < c->h.D; ++d) {
      if (lo) lo[d] = c->h.flo[d];
      if (hi) hi[d] = c->h.flo[d] < 0 ? -1 : c->h.flo[d] + c->h.fw[d] - 1;
    }
    if (nnz) *nnz = c->h.nnz();
  });
}

int pqdts_cuda_set_x(pqdts_ctx* c, const double* X) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    if (!X) throw Err(PQDTS_E_ARG, "null X");
    pqdts::set_x_colmajor(*c, X);
  });
}

int pqdts_cuda_get_x(pqdts_ctx* c, double* X) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    if (!X) throw Err(PQDTS_E_ARG, "null X");
    pqdts::get_x_colmajor(*c, X);
  });
}

int pqdts_cuda_init_x(pqdts_ctx* c) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    const int64_t MN = c->h.M * c->h.N;
    pqdts::k_fill<<<pqdts::elem_grid(MN), 256, 0, c->st>>>(MN, 1.0 / (double)c->h.N, c->X.p);
    pqdts::post_launch(*c);
    pqdts::touch_x(*c);
  });
}

int pqdts_cuda_get_stream(pqdts_ctx* c, void** stream) {
  if (!c || !stream) return PQDTS_E_ARG;
  *stream = (void*)c->st;
  return PQDTS_OK;
}

int pqdts_cuda_transfer_bytes(pqdts_ctx* c, int64_t* h2d, int64_t* d2h) {
  if (!c) return PQDTS_E_ARG;
  if (h2d) *h2d = c->h2d.load();
  if (d2h) *d2h = c->d2h.load();
  return PQDTS_OK;
}

int pqdts_cuda_set_space(pqdts_ctx* c, int32_t fullspace, const int32_t* maxr) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    if (fullspace) {
      c->fullspace = true;
      if (maxr) CK(cudaMemcpyAsync(c->maxr.p, maxr, c->h.M * 4, cudaMemcpyHostToDevice, c->st));
    } else {
      if (!maxr) throw Err(PQDTS_E_ARG, "reduced space needs maxr");
      for (int64_t j = 0; j < c->h.M; ++j)
        if (maxr[j] < 0 || maxr[j] >= c->h.N) throw Err(PQDTS_E_ARG, "maxr out of range");
      CK(cudaMemcpyAsync(c->maxr.p, maxr, c->h.M * 4, cudaMemcpyHostToDevice, c->st));
      c->fullspace = false;
    }
    pqdts::touch_x(*c);  // maxr and the space key the cached gradient
    CK(cudaStreamSynchronize(c->st));
  });
}

int pqdts_cuda_get_maxr(pqdts_ctx* c, int32_t* maxr) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    CK(cudaMemcpyAsync(maxr, c->maxr.p, c->h.M * 4, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  });
}

int pqdts_cuda_L(pqdts_ctx* c, double* val) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    *val = pqdts::op_L(*c);
  });
}

int pqdts_cuda_dL(pqdts_ctx* c, double* G) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    pqdts::op_dL(*c);
    pqdts::download_rowmajor_to_col(*c, c->G.p, G);
  });
}

int pqdts_cuda_redO(pqdts_ctx* c, double* O) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    const int64_t N = c->h.N, D = c->h.D;
    // R = 2*O - 0 via the Hessian epilogue, halved on the host (exact).
    pqdts::launch_fwd<double, 1>(*c, c->fval.p, c->X.p, 0, nullptr, c->R.p, 1, nullptr);
    c->R_ver = -1;  // R now holds 2*O, not 2*(O - P)
    CK(cudaMemcpyAsync(O, c->R.p, (size_t)D * N * 8, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (size_t k = 0; k < (size_t)D * N; ++k) O[k] *= 0.5;
  });
}

int pqdts_cuda_BF(pqdts_ctx* c, const double* V, double* HV) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    const int64_t M = c->h.M, N = c->h.N;
    std::vector<double> rm((size_t)M * N);
    for (int64_t i = 0; i < M; ++i)
      for (int64_t n = 0; n < N; ++n) rm[(size_t)i * N + n] = V[i + n * M];
    auto& b = c->cg64;
    CK(cudaMemcpyAsync(b.p.p, rm.data(), rm.size() * 8, cudaMemcpyHostToDevice, c->st));
    if (!c->fullspace) {
      pqdts::k_cg_lift<double><<<pqdts::cdiv(M, 32), pqdts::kLiftThreads, 0, c->st>>>(
          nullptr, 0, (int)M, (int)N, b.p.p, b.z.p, c->maxr.p, b.V.p, b.rs.p);
      pqdts::post_launch(*c);
    }
    pqdts::hvp<double>(*c, b, c->fval.p, c->tval.p, nullptr, false);
    pqdts::download_rowmajor_to_col(*c, b.Hp.p, HV);
  });
}

int pqdts_cuda_BF32(pqdts_ctx* c, const double* V, double* HV) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    if (c->precision != PQDTS_MIXED) throw Err(PQDTS_E_STATE, "BF32 needs a mixed-precision problem");
    const int64_t M = c->h.M, N = c->h.N;
    std::vector<float> rm((size_t)M * N);
    for (int64_t i = 0; i < M; ++i)
      for (int64_t n = 0; n < N; ++n) rm[(size_t)i * N + n] = (float)V[i + n * M];
    auto& b = c->cg32;
    CK(cudaMemcpyAsync(b.p.p, rm.data(), rm.size() * 4, cudaMemcpyHostToDevice, c->st));
    c->h2d += (int64_t)rm.size() * 4;
    if (!c->fullspace) {
      pqdts::k_cg_lift32<<<pqdts::cdiv(M * 32, 256), 256, 0, c->st>>>(nullptr, 0, (int)M, (int)N, b.p.p, b.z.p,
                                                                     c->maxr.p, b.V.p, b.rs.p);
      pqdts::post_launch(*c);
    }
    pqdts::hvp32(*c, b, nullptr, false, nullptr);
    CK(cudaMemcpyAsync(rm.data(), b.Hp.p, rm.size() * 4, cudaMemcpyDeviceToHost, c->st));
    pqdts::read_back(*c, c->sc.p, pqdts::SC_NSC);
    pqdts::check_tc_error(*c);
    c->d2h += (int64_t)rm.size() * 4;
    for (int64_t i = 0; i < M; ++i)
      for (int64_t n = 0; n < N; ++n) HV[i + n * M] = rm[(size_t)i * N + n];
  });
}

int pqdts_cuda_pdot(pqdts_ctx* c, const double* A, const double* B, double* out) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    const int64_t M = c->h.M, N = c->h.N;
    std::vector<double> ra((size_t)M * N), rb((size_t)M * N);
    for (int64_t i = 0; i < M; ++i)
      for (int64_t n = 0; n < N; ++n) {
        ra[(size_t)i * N + n] = A[i + n * M];
        rb[(size_t)i * N + n] = B[i + n * M];
      }
    auto& b = c->cg64;
    CK(cudaMemcpyAsync(b.p.p, ra.data(), ra.size() * 8, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(b.z.p, rb.data(), rb.size() * 8, cudaMemcpyHostToDevice, c->st));
    pqdts::dot_dev(*c, b.p.p, b.z.p, c->sc.p + pqdts::SC_TMP);
    CK(cudaMemcpyAsync(out, c->sc.p + pqdts::SC_TMP, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  });
}

int pqdts_cuda_Bdiag(pqdts_ctx* c, double* BD) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    const int64_t M = c->h.M, N = c->h.N;
    const double f = c->fullspace ? 1.0 : 2.0;
    for (int64_t n = 0; n < N; ++n)
      for (int64_t i = 0; i < M; ++i) BD[i + n * M] = c->h.bdiag[i] * f;
  });
}

int pqdts_cuda_doproj(pqdts_ctx* c) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    pqdts::project_rows(*c, c->X.p, nullptr, nullptr, c->X.p, 1);
    pqdts::touch_x(*c);
    CK(cudaStreamSynchronize(c->st));
  });
}

int pqdts_cuda_doproj2(pqdts_ctx* c, double* xmin) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    const int M = (int)c->h.M, N = (int)c->h.N;
    const int gb = pqdts::cdiv(M, 32);  // 32-row tiles
    pqdts::k_cand_proj2_t<<<dim3(gb, 1), pqdts::kTileThreads, 0, c->st>>>(c->X.p, nullptr, nullptr, c->X.p,
                                                                         (int64_t)M * N, c->maxr.p, M, N, 0,
                                                                         c->part2.p);
    pqdts::post_launch(*c);
    pqdts::touch_x(*c);
    pqdts::reduce_to(*c, c->part2.p, gb, c->sc.p + pqdts::SC_TMP, 1, true, 0.0);
    pqdts::read_back(*c, c->sc.p + pqdts::SC_TMP, 1);
    if (xmin) *xmin = c->pin[0];
  });
}

int pqdts_cuda_conv_test(pqdts_ctx* c, double* conv) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    *conv = pqdts::op_conv(*c, false);
  });
}

int pqdts_cuda_simplexproj(pqdts_ctx* c, const double* y, double* x, int64_t len, int64_t rows) {
  return guarded(c, [&] {
    if (!y || !x || len <= 0 || rows <= 0) throw Err(PQDTS_E_ARG, "bad simplexproj arguments");
    if (len * rows >= ((int64_t)1 << 31)) throw Err(PQDTS_E_ARG, "simplexproj input too large");
    pqdts::DBuf<double> d, w;
    d.alloc((size_t)(len * rows));
    w.alloc((size_t)(len * rows));
    CK(cudaMemcpyAsync(d.p, y, len * rows * 8, cudaMemcpyHostToDevice, c->st));
    pqdts::k_condat<<<dim3(pqdts::cdiv(rows, pqdts::kRowThreads), 1), pqdts::kRowThreads, 0, c->st>>>(
        d.p, nullptr, nullptr, d.p, w.p, 0, (int)rows, (int)len);
    pqdts::post_launch(*c);
    CK(cudaMemcpyAsync(x, d.p, len * rows * 8, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  });
}

// The reference's own projection symbol (condat_simplexproj.c:60, called
// from doproj at pqdts.f90:1133 through an implicit interface), so pqdts.f90
// links against this library unchanged.  Its signature has no context and
// no error return: each host thread (the reference calls it from OpenMP
// threads on private buffers) lazily gets its own stream and device buffers
// on the current device.  x receives the projection of y (x doubles as the
// reference's scratch; here y is copied to the device first, so x == y also
// gives the projection).  On a CUDA failure a message goes to stderr and x
// is filled with NaN, which the caller's objective then shows.
namespace pqdts {
struct CondatThreadState {
  int device = -1;
  cudaStream_t st = nullptr;
  double* buf = nullptr;  // 2 * cap doubles: the row, then Condat's working list
  int64_t cap = 0;
  void release() noexcept {
    if (buf) cudaFree(buf);
    if (st) cudaStreamDestroy(st);
    buf = nullptr;
    st = nullptr;
    cap = 0;
    device = -1;
  }
  ~CondatThreadState() { release(); }
};
static thread_local CondatThreadState t_condat;
}  // namespace pqdts

void simplexproj_condat_(double* y, double* x, int* plength) {
  if (!y || !x || !plength || *plength <= 0) return;
  const int len = *plength;
  pqdts::CondatThreadState& t = pqdts::t_condat;
  cudaError_t e = cudaSuccess;
  auto fail = [&](const char* what) {
    fprintf(stderr, "simplexproj_condat_: %s: %s\n", what, cudaGetErrorString(e));
    for (int i = 0; i < len; ++i) x[i] = std::numeric_limits<double>::quiet_NaN();
  };
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return fail("no current device");
  if (t.device != dev) {
    t.release();
    if ((e = cudaStreamCreateWithFlags(&t.st, cudaStreamNonBlocking)) != cudaSuccess) return fail("stream");
    t.device = dev;
  }
  if (t.cap < len) {
    if (t.buf) cudaFree(t.buf);
    t.buf = nullptr;
    t.cap = 0;
    if ((e = cudaMalloc((void**)&t.buf, (size_t)2 * len * sizeof(double))) != cudaSuccess) return fail("allocation");
    t.cap = len;
  }
  double* d = t.buf;
  double* w = t.buf + t.cap;
  if ((e = cudaMemcpyAsync(d, y, (size_t)len * 8, cudaMemcpyHostToDevice, t.st)) != cudaSuccess) return fail("upload");
  pqdts::k_condat<<<1, 32, 0, t.st>>>(d, nullptr, nullptr, d, w, 0, 1, len);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail("launch");
  if ((e = cudaMemcpyAsync(x, d, (size_t)len * 8, cudaMemcpyDeviceToHost, t.st)) != cudaSuccess) return fail("download");
  if ((e = cudaStreamSynchronize(t.st)) != cudaSuccess) return fail("projection");
}

int pqdts_cuda_smooth(int64_t M, int64_t N, double smo_fact, double* X) {
  if (M <= 0 || N <= 0 || !X || !(smo_fact > 0)) return PQDTS_E_ARG;
  try {
    // rows are independent: split them over host threads (same values)
    std::vector<double> Y(X, X + (size_t)M * N);
    auto rows = [&](int64_t j0, int64_t j1) {
      for (int64_t j = std::max<int64_t>(j0, 101); j < j1; ++j) {
        const int64_t dist = (int64_t)std::llround((double)j / smo_fact);
        const int64_t k0 = std::max<int64_t>(1, j - dist), k1 = std::min(j + dist, M);
        double rs = 0;
        for (int64_t i = 0; i < N; ++i) {
          double s = 0;
          int64_t c = 0;
          for (int64_t k = k0; k <= k1; ++k) {
            s = s + X[(k - 1) + i * M];
            c++;
          }
          Y[(j - 1) + i * M] = s / (double)c;
        }
        for (int64_t i = 0; i < N; ++i) rs += Y[(j - 1) + i * M];
        for (int64_t i = 0; i < N; ++i) Y[(j - 1) + i * M] = Y[(j - 1) + i * M] / rs;
      }
    };
    const int64_t nt = std::max<int64_t>(1, std::min<int64_t>(std::thread::hardware_concurrency(), (M + 255) / 256));
    std::vector<std::thread> pool;
    for (int64_t t = 0; t < nt; ++t) pool.emplace_back(rows, 1 + M * t / nt, 1 + M * (t + 1) / nt);
    for (auto& th : pool) th.join();
    std::copy(Y.begin(), Y.end(), X);
  } catch (const std::exception& e) {
    fprintf(stderr, "pqdts_cuda_smooth: %s\n", e.what());
    return PQDTS_E_STATE;
  }
  return PQDTS_OK;
}

int pqdts_cuda_simplexproj_noalloc(const double* d_y, double* d_x, int64_t len, int64_t rows, void* stream) {
  if (!d_y || !d_x || len <= 0 || rows <= 0) {
    fprintf(stderr, "pqdts_cuda_simplexproj_noalloc: null buffer or non-positive size\n");
    return PQDTS_E_ARG;
  }
  if (len > PQDTS_NOALLOC_SCRATCH / rows || len * rows > PQDTS_NOALLOC_SCRATCH) {
    fprintf(stderr,
            "pqdts_cuda_simplexproj_noalloc: rows*len = %lld*%lld exceeds the scratch capacity of %d values\n",
            (long long)rows, (long long)len, (int)PQDTS_NOALLOC_SCRATCH);
    return PQDTS_E_ARG;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= pqdts::kMaxDevices) {
    fprintf(stderr, "pqdts_cuda_simplexproj_noalloc: no usable current device: %s\n", cudaGetErrorString(e));
    return PQDTS_E_CUDA;
  }
  double* scratch = nullptr;
  {
    // set-up once per device (and context), with that device current: the
    // scratch's device address
    std::lock_guard<std::mutex> g(pqdts::g_noalloc_mu);
    pqdts::NoallocSlot& slot = pqdts::g_noalloc[dev];
    const unsigned long long id = pqdts::current_ctx_id();
    if (slot.ptr == nullptr || id == 0 || slot.ctx_id != id) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, pqdts::g_noalloc_scratch);
      if (e != cudaSuccess || p == nullptr) {
        fprintf(stderr, "pqdts_cuda_simplexproj_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
        slot.ptr = nullptr;
        return PQDTS_E_CUDA;
      }
      slot.ptr = static_cast<double*>(p);
      slot.ctx_id = pqdts::current_ctx_id();  // the lookup may have made the primary context current
    }
    scratch = slot.ptr;
  }
  pqdts::k_condat<<<dim3(pqdts::cdiv(rows, pqdts::kRowThreads), 1), pqdts::kRowThreads, 0, (cudaStream_t)stream>>>(
      d_y, nullptr, nullptr, d_x, scratch, 0, (int)rows, (int)len);
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "pqdts_cuda_simplexproj_noalloc: launch failed: %s\n", cudaGetErrorString(e));
    return PQDTS_E_CUDA;
  }
  return PQDTS_OK;
}

int pqdts_cuda_run_stage(pqdts_ctx* c, int32_t mode, int32_t oiter, int32_t maxiiter, double conv_thres,
                         int32_t output, double* stats) {
  return guarded(c, [&] {
    pqdts::need_problem(*c);
    if (mode != 1 && mode != 2) throw Err(PQDTS_E_ARG, "mode must be 1 or 2");
    if (oiter != 1 && oiter != 2) throw Err(PQDTS_E_ARG, "oiter must be 1 or 2");
    pqdts::SolveState st;
    c->n_cg = c->n_lsL = c->n_refine = 0;
    const double t0 = pqdts::wall();
    st.t0 = t0;
    pqdts::run_stage(*c, mode, oiter, maxiiter, conv_thres, output, st);
    if (c->precision == PQDTS_MIXED) pqdts::nonneg_x(*c, st);
    CK(cudaStreamSynchronize(c->st));
    pqdts::fill_stats(*c, st, pqdts::wall() - t0, stats);
  });
}

int pqdts_cuda_solve(pqdts_ctx* c, int32_t mode, int32_t maxiiter, double conv_thres, int32_t start_stage,
                     int32_t output, pqdts_stage_cb cb, void* user, double* stats) {
  return guarded(c, [&] { pqdts::solve(*c, mode, maxiiter, conv_thres, start_stage, output, cb, user, stats); });
}

int pqdts_cuda_set_objective_target(pqdts_ctx* c, double target) {
  if (!c) return PQDTS_E_ARG;
  c->target_L = target > 0 ? target : 0.0;
  return PQDTS_OK;
}

int pqdts_cuda_set_option(pqdts_ctx* c, const char* name, int64_t value) {
  return guarded(c, [&] {
    if (!name) throw pqdts::Err(PQDTS_E_ARG, "option name is null");
    const std::string n = name;
    if (n == "graphs") {
      c->use_graphs = value != 0;
    } else if (n == "autotune") {
      c->autotune = value != 0;
    } else if (n == "timers") {
      if (value < 0 || value > 2) throw pqdts::Err(PQDTS_E_ARG, "timers must be 0, 1 or 2");
      c->timers.enabled = value != 0;
      c->timers.detail = value == 2;
      c->drop_graphs();  // captured CG chunks carry their timer spans
    } else if (n == "rows_kernels") {
      if (value < -1 || value > 1) throw pqdts::Err(PQDTS_E_ARG, "rows_kernels must be -1, 0 or 1");
      c->rows_option = (int)value;
    } else if (n == "tc_splits1") {
      if (value < -1 || value == 0 || value > 8) throw pqdts::Err(PQDTS_E_ARG, "tc_splits1 must be -1 or 1..8");
      c->tc_splits1_option = (int)value;
    } else if (n == "tc_persistent") {
      if (value < -1 || value > 1) throw pqdts::Err(PQDTS_E_ARG, "tc_persistent must be -1, 0 or 1");
      c->tc_persistent_option = (int)value;
    } else if (n == "row_masks") {
      if (value < 0 || value > 1) throw pqdts::Err(PQDTS_E_ARG, "row_masks must be 0 or 1");
      c->mask_option = (int)value;
      c->drop_graphs();  // captured CG chunks hold the products' form
    } else if (n == "count_fmas") {
      if (value < 0 || value > 1) throw pqdts::Err(PQDTS_E_ARG, "count_fmas must be 0 or 1");
      c->count_fmas = value != 0;
      c->drop_graphs();
    } else if (n == "fmas.forward" || n == "fmas.transposed") {
      throw pqdts::Err(PQDTS_E_ARG, n + " is read-only");
    } else if (n == "tc_screen") {
      if (value < -1 || value > 1) throw pqdts::Err(PQDTS_E_ARG, "tc_screen must be -1, 0 or 1");
      c->tc_screen_option = (int)value;
    } else if (n == "tensor_cores") {
      if (value < -1 || value > 1) throw pqdts::Err(PQDTS_E_ARG, "tensor_cores must be -1, 0 or 1");
      c->tc_option = (int)value;
    } else if (n == "df_products") {
      if (value < -1 || value > 1) throw pqdts::Err(PQDTS_E_ARG, "df_products must be -1, 0 or 1");
      c->df_option = (int)value;
    } else if (n == "internal_f") {
      if (value < -1 || value > 1) throw pqdts::Err(PQDTS_E_ARG, "internal_f must be -1, 0 or 1");
      c->internal_f_option = (int)value;
    } else if (n == "fp64_refine") {
      if (value < 0 || value > 1) throw pqdts::Err(PQDTS_E_ARG, "fp64_refine must be 0 or 1");
      c->refine_option = (int)value;
    } else if (n == "tc_wait_ms") {
      if (value < 1 || value > 60000) throw pqdts::Err(PQDTS_E_ARG, "tc_wait_ms must be 1..60000");
      c->tc_wait_ns = (uint64_t)value * 1000000ull;
      c->drop_graphs();  // captured launches carry the old limit
    } else if (n == "tc_wait_probe") {
      if (value < 0 || value > 1) throw pqdts::Err(PQDTS_E_ARG, "tc_wait_probe must be 0 or 1");
      c->tc_wait_probe = (int)value;
      c->drop_graphs();
    } else if (n == "df_rows") {
      if (value != 0 && value != 2 && value != 4 && value != 8)
        throw pqdts::Err(PQDTS_E_ARG, "df_rows must be 0, 2, 4 or 8");
      c->df_rows = (int)value;
    } else {
      throw pqdts::Err(PQDTS_E_ARG, "unknown option " + n);
    }
  });
}

int pqdts_cuda_get_option(pqdts_ctx* c, const char* name, int64_t* value) {
  return guarded(c, [&] {
    if (!name || !value) throw pqdts::Err(PQDTS_E_ARG, "null argument");
    const std::string n = name;
    const pqdts::Schedule& s = c->sched;
    if (n == "graphs") *value = c->use_graphs;
    else if (n == "autotune") *value = c->autotune;
    else if (n == "timers") *value = c->timers.enabled ? (c->timers.detail ? 2 : 1) : 0;
    else if (n == "sched.fwd_tile") *value = s.fwd_tile;
    else if (n == "sched.trn_tile") *value = s.trn_tile;
    else if (n == "sched.trn_splits") *value = s.trn_splits;
    else if (n == "sched.trans_threads") *value = s.trans_threads;
    else if (n == "sched.trans_cols") *value = s.trans_cols;
    else if (n == "sched.tuned") *value = s.tuned;
    else if (n == "sched.tc") *value = s.tc;
    else if (n == "sched.tc_splits") *value = s.tc_splits;
    else if (n == "sched.tc_bn") *value = s.tc_bn;
    else if (n == "sched.tc_persistent") *value = s.tc_persistent;
    else if (n == "sched.tc_splits1") *value = s.tc_splits1;
    else if (n == "sched.fwd_rows") *value = s.fwd_rows;
    else if (n == "sched.trans_rows") *value = s.trans_rows;
    else if (n == "rows_kernels") *value = c->rows_option;
    else if (n == "tc_persistent") *value = c->tc_persistent_option;
    else if (n == "tc_screen") *value = c->tc_screen_option;
    else if (n == "row_masks") *value = c->mask_option;
    else if (n == "count_fmas") *value = c->count_fmas ? 1 : 0;
    else if (n == "fmas.forward" || n == "fmas.transposed") {
      unsigned long long v[2] = {0, 0};
      if (c->fmacount.p) {
        CK(cudaMemcpyAsync(v, c->fmacount.p, sizeof(v), cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
      }
      *value = (int64_t)(n == "fmas.forward" ? v[0] : v[1]);
    }
    else if (n == "tensor_cores") *value = c->tc_option;
    else if (n == "df_products") *value = c->df_option;
    else if (n == "df_rows") *value = c->df_rows;
    else if (n == "tc_wait_ms") *value = (int64_t)(c->tc_wait_ns / 1000000ull);
    else if (n == "tc_wait_probe") *value = c->tc_wait_probe;
    else if (n == "fp64_refine") *value = c->refine_option;
    else if (n == "internal_f") *value = c->internal_f_option;
    else if (n == "sched.df_fwd") *value = c->df_fwd;
    else if (n == "sched.df_trans") *value = c->df_trans;
    else if (n == "sched.tc_screen") *value = (s.tc && c->tc_ready && c->tc_screen_option != 0) ? 1 : 0;
    else if (n == "graphs.captured") *value = (int64_t)c->graphs.size();
    else throw pqdts::Err(PQDTS_E_ARG, "unknown option " + n);
  });
}

int pqdts_cuda_timer(pqdts_ctx* c, const char* name, double* seconds, int64_t* count) {
  return guarded(c, [&] {
    c->timers.flush();
    for (size_t i = 0; i < c->timers.names.size(); ++i)
      if (c->timers.names[i] == name) {
        if (seconds) *seconds = c->timers.secs[i];
        if (count) *count = c->timers.counts[i];
        return;
      }
    if (seconds) *seconds = 0;
    if (count) *count = 0;
  });
}

// Tasks of a batched solve: single instances, and groups of instances that
// share F (the same M, N, D and bands and values) solved in lockstep with a
// joint CG (mixed precision, mode 2, N <= kGroupMaxN; at most kGroupMax
// members and M*G*N < 2^31 per group), when PQDTS_BATCH_GROUPS=1 turns the
// grouping on.  It is off by default: a group's members take their line
// searches one after another on the group's worker and its joint CG runs
// as long as its slowest member's, and on the 64-instance batch (8
// detectors x 8 resamples) the groups took 6.4 s (16 groups of 4 on 16
// workers; 6.9 s as 8 groups of 8) against 5.0 s for 64 independent solves
// on 16 workers.
static constexpr int kGroupMax = 4;
static constexpr int64_t kGroupMaxN = 4096;

static std::vector<std::vector<int>> batch_tasks(int n_inst, const int64_t* M, const int64_t* N, const int64_t* D,
                                                 const int64_t* band_lo, const int64_t* band_hi,
                                                 const double* band_vals, const int64_t* band_row_offset,
                                                 const int64_t* band_val_offset, bool grouping) {
  std::vector<std::vector<int>> tasks;
  if (!grouping) {
    for (int k = 0; k < n_inst; ++k) tasks.push_back({k});
    return tasks;
  }
  auto nvals = [&](int k) {
    int64_t t = 0;
    for (int64_t d = 0; d < D[k]; ++d)
      if (band_lo[band_row_offset[k] + d] >= 0) t += band_hi[band_row_offset[k] + d] - band_lo[band_row_offset[k] + d] + 1;
    return t;
  };
  auto fnv = [](uint64_t h, const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 0x100000001B3ULL;
    return h;
  };
  std::vector<int64_t> nv(n_inst);
  std::map<uint64_t, std::vector<int>> buckets;
  std::vector<uint64_t> key(n_inst);
  for (int k = 0; k < n_inst; ++k) {
    nv[k] = nvals(k);
    uint64_t h = 0xCBF29CE484222325ULL;
    const int64_t shape[4] = {M[k], N[k], D[k], nv[k]};
    h = fnv(h, shape, sizeof(shape));
    h = fnv(h, band_lo + band_row_offset[k], (size_t)D[k] * 8);
    h = fnv(h, band_hi + band_row_offset[k], (size_t)D[k] * 8);
    h = fnv(h, band_vals + band_val_offset[k], (size_t)nv[k] * 8);
    key[k] = h;
    buckets[h].push_back(k);
  }
  auto same = [&](int a, int b) {
    return M[a] == M[b] && N[a] == N[b] && D[a] == D[b] && nv[a] == nv[b] &&
           std::memcmp(band_lo + band_row_offset[a], band_lo + band_row_offset[b], (size_t)D[a] * 8) == 0 &&
           std::memcmp(band_hi + band_row_offset[a], band_hi + band_row_offset[b], (size_t)D[a] * 8) == 0 &&
           std::memcmp(band_vals + band_val_offset[a], band_vals + band_val_offset[b], (size_t)nv[a] * 8) == 0;
  };
  std::vector<char> taken(n_inst, 0);
  for (int k = 0; k < n_inst; ++k) {
    if (taken[k]) continue;
    std::vector<int> grp{k};
    taken[k] = 1;
    for (int j : buckets[key[k]])
      if (!taken[j] && same(k, j)) {
        grp.push_back(j);
        taken[j] = 1;
      }
    const int64_t cap = std::max<int64_t>(1, std::min<int64_t>(kGroupMax, (((int64_t)1 << 31) - 1) / (M[k] * N[k])));
    const bool joint = grp.size() >= 2 && N[k] <= kGroupMaxN && cap >= 2;
    if (!joint) {
      for (int j : grp) tasks.push_back({j});
      continue;
    }
    // equal parts of at most `cap` members
    const int64_t parts = ((int64_t)grp.size() + cap - 1) / cap;
    size_t at = 0;
    for (int64_t q = 0; q < parts; ++q) {
      const size_t n = (grp.size() - at) / (size_t)(parts - q);
      tasks.emplace_back(grp.begin() + at, grp.begin() + at + n);
      at += n;
    }
  }
  return tasks;
}

int pqdts_cuda_batch_groups(int32_t n_inst, const int64_t* M, const int64_t* N, const int64_t* D,
                            const int64_t* band_lo, const int64_t* band_hi, const double* band_vals,
                            const int64_t* band_row_offset, const int64_t* band_val_offset, int32_t* group_of) {
  if (n_inst <= 0 || !M || !N || !D || !band_lo || !band_hi || !band_vals || !band_row_offset || !band_val_offset ||
      !group_of)
    return PQDTS_E_ARG;
  try {
    const auto tasks = batch_tasks(n_inst, M, N, D, band_lo, band_hi, band_vals, band_row_offset, band_val_offset, true);
    for (size_t t = 0; t < tasks.size(); ++t)
      for (int k : tasks[t]) group_of[k] = tasks[t].size() >= 2 ? (int32_t)t : -1;
  } catch (const std::exception& e) {
    fprintf(stderr, "pqdts_cuda_batch_groups: %s\n", e.what());
    return PQDTS_E_STATE;
  }
  return PQDTS_OK;
}

int pqdts_cuda_solve_batch(int32_t device, int32_t n_inst, const int64_t* M, const int64_t* N, const int64_t* D,
                           const int64_t* band_lo, const int64_t* band_hi, const double* band_vals,
                           const int64_t* band_row_offset, const int64_t* band_val_offset, const double* P,
                           const int64_t* P_offset, const double* gamma, int32_t precision, int32_t mode,
                           int32_t maxiiter, double conv_thres, const double* target_L, double* X,
                           double* stats) {
  if (n_inst <= 0 || !M || !N || !D || !band_lo || !band_hi || !band_vals || !band_row_offset || !band_val_offset ||
      !P || !P_offset || !gamma || !X)
    return PQDTS_E_ARG;
  // Tasks are independent: a pool of host workers, each with its own
  // context and stream, so the tasks' kernels overlap on the device.
  std::vector<int64_t> xoff(n_inst + 1, 0);
  for (int k = 0; k < n_inst; ++k) xoff[k + 1] = xoff[k] + M[k] * N[k];
  bool grouping = false;
  if (const char* e = std::getenv("PQDTS_BATCH_GROUPS")) grouping = precision == PQDTS_MIXED && mode == 2 && std::atoi(e) != 0;
  std::vector<std::vector<int>> tasks;
  try {
    tasks = batch_tasks(n_inst, M, N, D, band_lo, band_hi, band_vals, band_row_offset, band_val_offset, grouping);
  } catch (const std::exception& e) {
    fprintf(stderr, "pqdts_cuda_solve_batch: %s\n", e.what());
    return PQDTS_E_STATE;
  }
  const int ntask = (int)tasks.size();
  // workers: PQDTS_BATCH_WORKERS (default: the host's hardware threads, at
  // most 16), at most one per task
  int workers = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (const char* e = std::getenv("PQDTS_BATCH_WORKERS")) workers = std::max(1, std::min(64, std::atoi(e)));
  workers = std::min<int>(ntask, workers);
  std::atomic<int> next{0};
  std::atomic<int> rc{PQDTS_OK};
  std::mutex err_mu;
  auto fail = [&](int k, pqdts_ctx* c, int r) {
    std::lock_guard<std::mutex> g(err_mu);
    fprintf(stderr, "pqdts_cuda_solve_batch: instance %d: %s\n", k, c ? c->err.c_str() : "context creation failed");
    rc = r;
  };
  auto setup = [&](pqdts_ctx* c, int k) {
    const int64_t* lo = band_lo + band_row_offset[k];
    const int64_t* hi = band_hi + band_row_offset[k];
    int r = pqdts_cuda_set_problem(c, M[k], N[k], D[k], lo, hi, band_vals + band_val_offset[k], P + P_offset[k],
                                   gamma[k], precision);
    if (r == PQDTS_OK) r = pqdts_cuda_set_x(c, X + xoff[k]);
    if (r == PQDTS_OK) r = pqdts_cuda_set_objective_target(c, target_L ? target_L[k] : 0.0);
    return r;
  };
  auto single = [&](pqdts_ctx* c, int k) {
    int r = setup(c, k);
    if (r == PQDTS_OK)
      r = pqdts_cuda_solve(c, mode, maxiiter, conv_thres, 1, 0, nullptr, nullptr,
                           stats ? stats + (int64_t)k * PQDTS_NSTATS : nullptr);
    if (r == PQDTS_OK) r = pqdts_cuda_get_x(c, X + xoff[k]);
    if (r != PQDTS_OK) fail(k, c, r);
  };
  // A group: the widened problem (M, G*N, D, the shared F; P and gamma are
  // not used) on a group context whose stream the members share; members
  // fall back to single solves when the group cannot take the joint CG.
  auto group = [&](pqdts_ctx* c, const std::vector<int>& ks) {
    const int G = (int)ks.size(), k0 = ks[0];
    pqdts_ctx* g = nullptr;
    int r = pqdts_cuda_create(device, &g);
    if (r == PQDTS_OK) {
      g->timers.enabled = false;
      std::vector<double> Pz((size_t)D[k0] * N[k0] * G, 0.0);
      r = pqdts_cuda_set_problem(g, M[k0], N[k0] * G, D[k0], band_lo + band_row_offset[k0],
                                 band_hi + band_row_offset[k0], band_vals + band_val_offset[k0], Pz.data(), 0.0,
                                 precision);
    }
    if (r != PQDTS_OK || !pqdts::group_ready(*g, N[k0])) {
      if (g) pqdts_cuda_destroy(g);
      for (int k : ks)
        if (rc.load() == PQDTS_OK) single(c, k);
      return;
    }
    std::vector<pqdts_ctx*> mc(G, nullptr);
    std::vector<pqdts::MemberRun> ms(G);
    for (int j = 0; j < G && r == PQDTS_OK; ++j) {
      r = create_ctx(device, g->st, &mc[j]);
      if (r != PQDTS_OK) {
        fail(ks[j], nullptr, r);
        break;
      }
      mc[j]->timers.enabled = false;
      mc[j]->tc_option = 0;  // the members' own CG products are not used
      r = setup(mc[j], ks[j]);
      if (r != PQDTS_OK) fail(ks[j], mc[j], r);
      ms[j].c = mc[j];
      ms[j].maxiiter = maxiiter;
      ms[j].conv_thres = conv_thres;
      ms[j].stats = stats ? stats + (int64_t)ks[j] * PQDTS_NSTATS : nullptr;
    }
    if (r == PQDTS_OK) {
      r = guarded(g, [&] { pqdts::group_solve(*g, ms); });
      if (r != PQDTS_OK) fail(k0, g, r);
    }
    for (int j = 0; j < G && r == PQDTS_OK; ++j) {
      r = pqdts_cuda_get_x(mc[j], X + xoff[ks[j]]);
      if (r != PQDTS_OK) fail(ks[j], mc[j], r);
    }
    for (pqdts_ctx* m : mc)
      if (m) pqdts_cuda_destroy(m);
    pqdts_cuda_destroy(g);
  };
  auto work = [&]() {
    pqdts_ctx* c = nullptr;
    int r = pqdts_cuda_create(device, &c);
    if (r != PQDTS_OK) {
      rc = r;
      return;
    }
    c->timers.enabled = false;  // no per-region events in the batch
    for (;;) {
      const int t = next++;
      if (t >= ntask || rc.load() != PQDTS_OK) break;
      if (tasks[t].size() == 1) single(c, tasks[t][0]);
      else group(c, tasks[t]);
    }
    pqdts_cuda_destroy(c);
  };
  std::vector<std::thread> th;
  for (int w = 0; w < workers; ++w) th.emplace_back(work);
  for (auto& t : th) t.join();
  return rc.load();
}

}  // extern "C"
