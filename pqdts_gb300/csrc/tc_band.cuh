// Banded products on the 5th-generation tensor cores (tcgen05 + TMA) with
// split-BF16x3 compensation: every FP32 operand x is held as the bf16 pair
// hi = bf16(x), lo = bf16(x - hi), and a product a.b is accumulated in FP32
// as hi_a.hi_b + hi_a.lo_b + lo_a.hi_b (the lo.lo term, ~2^-16 relative,
// is dropped).  Used for the Hessian-vector products of the mixed-precision
// CG (BF, pqdts.f90:246-342), whose FP32 accumulation it replaces.
//
// Out[r, n] = scale * sum_k Band[r, k] * B[n, k]
//
// The band operand is stored in 128-row blocks, each with its own K window
// [kb, kb + kTcK*nch) (kb a multiple of kTcK = 32, zero filled outside the
// rows' bands): rows r of block b hold Band[r, kb + x] at local column x.  B
// is N rows of K (K contiguous, "K-major"): V^T for F.V, (2 F.V)^T for
// F^T.(.).  One CTA computes a 128 x BN tile: warp 0 lane 0 streams 32-wide
// K chunks of A hi/lo and B hi/lo through a ring of up to 6 shared-memory
// stages with TMA (64-byte rows, 64-byte swizzle: a BN = 256 stage is 48 KB,
// so 4 stages fit beside the epilogue), warp 1 lane 0 issues the MMAs (M=128, N=BN, K=16,
// bf16 in, FP32 accumulator in tensor memory), all four warps then read the
// accumulator back (tcgen05.ld, one row per thread) and store it.
//
// Every mbarrier wait is bounded (wait_ns, by default kTcWaitNs); a wait
// that runs out sets *err, skips the remaining work and stores nothing, and
// the CTA frees its tensor memory only after the copies in flight have
// landed and the MMAs already issued have completed (the issuer's last
// tcgen05.commit).  `probe` != 0 is a test hook: the producer first waits on
// a barrier that nothing arrives on, so the wait runs out before any copy or
// MMA is issued and the error path runs on an otherwise valid launch.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cstdint>

namespace pqdts {

constexpr int kTcThreads = 128;
constexpr int kTcRows = 128;           // rows of a band block = MMA M
constexpr int kTcK = 32;               // K per stage: one 64-byte swizzled row of bf16
constexpr uint32_t kTcRowBytes = kTcK * 2;  // bytes of one operand row in a stage
constexpr int kTcMaxStages = 6;
static_assert(kTcRowBytes == 32 || kTcRowBytes == 64 || kTcRowBytes == 128, "swizzle width");
constexpr uint64_t kTcWaitNs = 2000000000ull;  // 2 s per wait (default)

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Wait for the phase of `parity` to complete; false when limit_ns ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}

// 2-D TMA tile load (x = inner coordinate, elements) completing on `bar`.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
          "r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Fetch a TMA descriptor ahead of its first use (overlaps the set-up).
__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
}

__device__ __forceinline__ void tc_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tc_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D(tmem) (+)= A(smem) . B(smem)^T, kind::f16 (bf16 inputs, FP32 accumulator).
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive on `bar` once all tcgen05 operations issued so far have completed.
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// 16 consecutive FP32 columns of this thread's accumulator row (32x32b
// shape: lane t of the warp reads TMEM lane base + t), waited in place.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// Shared-memory matrix descriptor of a K-major operand tile written by TMA
// with the swizzle of its row width (kTcRowBytes = 128, 64 or 32 bytes):
// 8-row groups 8 * kTcRowBytes apart (stride byte offset), tile base aligned
// to 1024 bytes; advancing the start address by 32 bytes selects the next
// K=16 slice of the swizzled row.  Layout field (bits 61-63): 2 = 128-byte,
// 4 = 64-byte, 6 = 32-byte swizzle.
__device__ __forceinline__ uint64_t swz_desc(uint32_t saddr) {
  constexpr uint64_t layout = kTcRowBytes == 128 ? 2 : kTcRowBytes == 64 ? 4 : 6;
  return (uint64_t)((saddr & 0x3FFFFu) >> 4)           // start address
         | ((uint64_t)1 << 16)                         // leading byte offset (unused for swizzled K-major)
         | ((uint64_t)((8 * kTcRowBytes) >> 4) << 32)  // stride byte offset
         | ((uint64_t)1 << 46)                         // descriptor version
         | (layout << 61);                             // swizzle mode
}

// Instruction descriptor, kind::f16: FP32 accumulator, bf16 A and B, both
// K-major, M x N.
__host__ __device__ constexpr uint32_t tc_idesc_bf16(int m, int n) {
  return (1u << 4)                          // D format: F32
         | (1u << 7)                        // A format: BF16
         | (1u << 10)                       // B format: BF16
         | ((uint32_t)(n >> 3) << 17)       // N / 8
         | ((uint32_t)(m >> 4) << 24);      // M / 16
}

__host__ __device__ constexpr uint32_t tc_tmem_cols(int bn) {
  return bn <= 32 ? 32u : bn <= 64 ? 64u : bn <= 128 ? 128u : 256u;
}

// mode 0: FP32 Out[z * out_stride + r * N + n] = scale * acc (row-major; z =
//         the K split whose partial this is).
// mode 1: Out^T split again: oh[n * ld + r] = hi, ol[n * ld + r] = lo of
//         scale * acc (the next product's K-major B operand).
__global__ void __launch_bounds__(kTcThreads, 1)
    k_tc_band(const __grid_constant__ CUtensorMap mA_hi, const __grid_constant__ CUtensorMap mA_lo,
              const __grid_constant__ CUtensorMap mB_hi, const __grid_constant__ CUtensorMap mB_lo,
              const int32_t* __restrict__ blk_kb, const int32_t* __restrict__ blk_nch, int R, int N, int BN,
              int stages, int splits, int mode, float scale, float* __restrict__ out, int64_t out_stride,
              __nv_bfloat16* __restrict__ oh, __nv_bfloat16* __restrict__ ol, int64_t ld,
              const double* __restrict__ pred, double* __restrict__ err, uint64_t wait_ns, int probe) {
  if (pred != nullptr && pred[6] != 0.0) return;  // CG already converged
  extern __shared__ uint8_t tc_smem_raw[];
  __shared__ uint64_t bar_full[kTcMaxStages], bar_empty[kTcMaxStages], bar_acc, bar_probe;
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  __shared__ int s_issued, s_consumed;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int blk = blockIdx.y, n0 = blockIdx.x * BN, r0 = blk * kTcRows;
  const int kb = blk_kb[blk];
  int c0 = 0, c1 = kb >= 0 ? blk_nch[blk] : 0;
  if (splits > 1) {  // this CTA's share of the block's K chunks
    const int per = (c1 + splits - 1) / splits;
    c0 = min(c1, (int)blockIdx.z * per);
    c1 = min(c1, c0 + per);
  }
  const int nk = c1 - c0;

  // stage ring, 1024-byte aligned (swizzle atoms)
  const uint32_t raw = smem_u32(tc_smem_raw);
  uint8_t* base = tc_smem_raw + ((1024u - (raw & 1023u)) & 1023u);
  const uint32_t a_bytes = kTcRows * kTcRowBytes, b_bytes = (uint32_t)BN * kTcRowBytes;
  const uint32_t stage_bytes = 2u * a_bytes + 2u * b_bytes;

  if (threadIdx.x == 0) {
    tma_prefetch_desc(&mA_hi);
    tma_prefetch_desc(&mA_lo);
    tma_prefetch_desc(&mB_hi);
    tma_prefetch_desc(&mB_lo);
    for (int i = 0; i < stages; ++i) {
      mbar_init(&bar_full[i], 1);
      mbar_init(&bar_empty[i], 1);
    }
    mbar_init(&bar_acc, 1);
    mbar_init(&bar_probe, 1);
    s_abort = 0;
    s_issued = 0;
    s_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  const uint32_t ncols = tc_tmem_cols(BN);
  if (warp == 0) {
    tc_alloc(&s_tmem, ncols);
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;

  if (warp == 0 && lane == 0 && nk > 0) {
    // producer: TMA loads of A hi/lo (block-local K) and B hi/lo (global K)
    if (probe && !mbar_wait(&bar_probe, 0, wait_ns)) s_abort = 1;  // nothing arrives: runs out
    for (int it = 0; it < nk && !s_abort; ++it) {
      const int st = it % stages;
      const uint32_t ph = (uint32_t)(it / stages) & 1u;
      if (!mbar_wait(&bar_empty[st], ph ^ 1u, wait_ns)) {
        s_abort = 1;
        break;
      }
      uint8_t* sa = base + (size_t)st * stage_bytes;
      uint8_t* sb = sa + 2 * a_bytes;
      mbar_expect_tx(&bar_full[st], stage_bytes);
      const int kx = (c0 + it) * kTcK;
      tma_load_2d(sa, &mA_hi, kx, r0, &bar_full[st]);
      tma_load_2d(sa + a_bytes, &mA_lo, kx, r0, &bar_full[st]);
      tma_load_2d(sb, &mB_hi, kb + kx, n0, &bar_full[st]);
      tma_load_2d(sb + b_bytes, &mB_lo, kb + kx, n0, &bar_full[st]);
      s_issued = it + 1;
    }
  } else if (warp == 1 && lane == 0 && nk > 0) {
    // MMA issuer: 4 K-slices of 16 x 3 compensated terms per stage
    const uint32_t idesc = tc_idesc_bf16(kTcRows, BN);
    for (int it = 0; it < nk && !s_abort; ++it) {
      const int st = it % stages;
      const uint32_t ph = (uint32_t)(it / stages) & 1u;
      if (!mbar_wait(&bar_full[st], ph, wait_ns)) {
        s_abort = 1;
        break;
      }
      s_consumed = it + 1;
      tc_fence_after();
      const uint32_t a_hi = smem_u32(base + (size_t)st * stage_bytes);
      const uint32_t a_lo = a_hi + a_bytes, b_hi = a_hi + 2 * a_bytes, b_lo = b_hi + b_bytes;
#pragma unroll
      for (int k = 0; k < kTcK / 16; ++k) {
        const uint32_t o = 32u * k;
        tc_mma(tmem, swz_desc(a_lo + o), swz_desc(b_hi + o), idesc, (it > 0 || k > 0) ? 1u : 0u);
        tc_mma(tmem, swz_desc(a_hi + o), swz_desc(b_lo + o), idesc, 1u);
        tc_mma(tmem, swz_desc(a_hi + o), swz_desc(b_hi + o), idesc, 1u);
      }
      tc_commit(&bar_empty[st]);  // the stage is free once these MMAs are done
    }
    tc_commit(&bar_acc);  // also after an abort: arrives once every issued MMA is done
  }
  __syncwarp();

  // epilogue: thread t of warp w owns accumulator row 32w + t
  bool ok = true;
  if (nk > 0) {
    ok = mbar_wait(&bar_acc, 0, wait_ns);
    tc_fence_after();
  }
  if (!ok) s_abort = 1;
  const int r = r0 + warp * 32 + lane;
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
  // the warp's decision (uniform: the loads below are warp-collective)
  const bool store = __all_sync(0xffffffffu, ok && !s_abort);
  if (mode == 0) {
    // FP32 rows: staged through the (now idle) stage ring so each store
    // instruction writes 128 contiguous bytes of one row; warp w uses rows
    // 32w..32w+31 of the tile, row stride = 1 mod 32 words (no bank conflicts)
    const int stride = BN + ((33 - BN % 32) % 32);
    float* mine = reinterpret_cast<float*>(base) + (size_t)(warp * 32) * stride;
    for (int cc = 0; cc < BN; cc += 16) {
      float v[16];
      if (nk > 0) {
        tc_ld16(trow + (uint32_t)cc, v);
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = 0.f;
      }
      if (store) {
#pragma unroll
        for (int j = 0; j < 16; ++j) mine[lane * stride + cc + j] = v[j];
      }
    }
    __syncwarp();
    if (store) {
      float* o = out + (int64_t)blockIdx.z * out_stride;
      for (int rr = 0; rr < 32; ++rr) {
        const int row = r0 + warp * 32 + rr;
        if (row >= R) break;
        for (int x = lane; x < BN; x += 32) {
          const int n = n0 + x;
          if (n < N) o[(int64_t)row * N + n] = scale * mine[rr * stride + x];
        }
      }
    }
  } else {
    // (F.V)^T split: for each column n the warp writes 32 consecutive rows
    for (int cc = 0; cc < BN; cc += 16) {
      float v[16];
      if (nk > 0) {
        tc_ld16(trow + (uint32_t)cc, v);
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = 0.f;
      }
      if (store && r < R) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const int n = n0 + cc + j;
          if (n < N) {
            const float x = scale * v[j];
            const __nv_bfloat16 h = __float2bfloat16_rn(x);
            oh[(int64_t)n * ld + r] = h;
            ol[(int64_t)n * ld + r] = __float2bfloat16_rn(x - __bfloat162float(h));
          }
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (s_abort && threadIdx.x == 0) {
    *err = 1.0;
    // let the copies already in flight land before the CTA's memory goes
    for (int it = s_consumed; it < s_issued; ++it)
      if (!mbar_wait(&bar_full[it % stages], (uint32_t)(it / stages) & 1u, wait_ns)) break;
    // and the MMAs already issued finish with tensor and shared memory
    // (the issuer committed bar_acc after its last one, aborted or not)
    if (nk > 0) mbar_wait(&bar_acc, 0, wait_ns);
  }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tc_dealloc(tmem, ncols);
  }
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Persistent form of k_tc_band (same operands, modes and results): one CTA
// per SM walks its list of output tiles sched_tile[sched_off[b] ..
// sched_off[b+1]) (tile t: N tile t % ntn, then row block, then K split;
// the host balances the lists by each tile's K chunks, longest first), or
// with sched_off = null t = blockIdx.x, blockIdx.x + gridDim.x, ...  Six warps: warp 0
// lane 0 issues the TMA loads, warp 1 lane 0 the MMAs (warp 1 owns the
// tensor memory), warps 2-5 run the epilogue.  Two FP32 accumulators in
// tensor memory let the epilogue of tile j overlap the MMAs of tile j+1,
// and the shared-memory stage ring runs on across tiles.
constexpr int kTcpThreads = 192;

__global__ void __launch_bounds__(kTcpThreads, 1)
    k_tc_band_p(const __grid_constant__ CUtensorMap mA_hi, const __grid_constant__ CUtensorMap mA_lo,
                const __grid_constant__ CUtensorMap mB_hi, const __grid_constant__ CUtensorMap mB_lo,
                const int32_t* __restrict__ blk_kb, const int32_t* __restrict__ blk_nch, int R, int N, int BN,
                int stages, int splits, int blocks, int mode, float scale, float* __restrict__ out,
                int64_t out_stride, __nv_bfloat16* __restrict__ oh, __nv_bfloat16* __restrict__ ol, int64_t ld,
                const double* __restrict__ pred, double* __restrict__ err, uint64_t wait_ns, int probe,
                const int32_t* __restrict__ sched_off, const int32_t* __restrict__ sched_tile) {
  if (pred != nullptr && pred[6] != 0.0) return;  // CG already converged
  extern __shared__ uint8_t tc_smem_raw[];
  __shared__ uint64_t bar_full[kTcMaxStages], bar_empty[kTcMaxStages], bar_tfull[2], bar_tempty[2], bar_fin,
      bar_probe;
  __shared__ uint32_t s_tmem;
  __shared__ volatile int s_abort;
  __shared__ int s_issued, s_consumed;
  __shared__ float s_stage[4][32][17];  // epilogue staging of mode 0, one 32 x 16 slab per warp

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntn = (N + BN - 1) / BN;
  const int T = ntn * blocks * splits;
  const uint32_t raw = smem_u32(tc_smem_raw);
  uint8_t* base = tc_smem_raw + ((1024u - (raw & 1023u)) & 1023u);
  const uint32_t a_bytes = kTcRows * kTcRowBytes, b_bytes = (uint32_t)BN * kTcRowBytes;
  const uint32_t stage_bytes = 2u * a_bytes + 2u * b_bytes;
  const uint32_t ncols = tc_tmem_cols(BN);  // per accumulator

  if (threadIdx.x == 0) {
    tma_prefetch_desc(&mA_hi);
    tma_prefetch_desc(&mA_lo);
    tma_prefetch_desc(&mB_hi);
    tma_prefetch_desc(&mB_lo);
    for (int i = 0; i < stages; ++i) {
      mbar_init(&bar_full[i], 1);
      mbar_init(&bar_empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&bar_tfull[i], 1);
      mbar_init(&bar_tempty[i], 128);
    }
    mbar_init(&bar_fin, 1);
    mbar_init(&bar_probe, 1);
    s_abort = 0;
    s_issued = 0;
    s_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    tc_alloc(&s_tmem, 2 * ncols);
    tc_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;

  // this CTA's tiles: entries [j_begin, j_end) of its list (or the
  // round-robin sequence blockIdx.x + j * gridDim.x)
  const int j_begin = sched_off ? sched_off[blockIdx.x] : 0;
  const int j_end = sched_off ? sched_off[blockIdx.x + 1] : (T - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
  auto tile_of = [&](int j) { return sched_off ? sched_tile[j] : (int)blockIdx.x + j * (int)gridDim.x; };
  // tile t -> N tile, row block, K chunk range [c0, c1), block K start kb
  auto tile = [&](int t, int& nt, int& blk, int& c0, int& c1, int& kb) {
    nt = t % ntn;
    const int rest = t / ntn;
    blk = rest % blocks;
    const int sp = rest / blocks;
    kb = blk_kb[blk];
    c0 = 0;
    c1 = kb >= 0 ? blk_nch[blk] : 0;
    if (splits > 1) {
      const int per = (c1 + splits - 1) / splits;
      c0 = min(c1, sp * per);
      c1 = min(c1, c0 + per);
    }
  };

  if (warp == 0) {
    if (lane == 0) {
      int it = 0;
      if (probe && !mbar_wait(&bar_probe, 0, wait_ns)) s_abort = 1;  // nothing arrives: runs out
      for (int j = j_begin; j < j_end && !s_abort; ++j) {
        int nt, blk, c0, c1, kb;
        tile(tile_of(j), nt, blk, c0, c1, kb);
        for (int ch = c0; ch < c1 && !s_abort; ++ch, ++it) {
          const int st = it % stages;
          const uint32_t ph = (uint32_t)(it / stages) & 1u;
          if (!mbar_wait(&bar_empty[st], ph ^ 1u, wait_ns)) {
            s_abort = 1;
            break;
          }
          uint8_t* sa = base + (size_t)st * stage_bytes;
          uint8_t* sb = sa + 2 * a_bytes;
          mbar_expect_tx(&bar_full[st], stage_bytes);
          const int kx = ch * kTcK;
          tma_load_2d(sa, &mA_hi, kx, blk * kTcRows, &bar_full[st]);
          tma_load_2d(sa + a_bytes, &mA_lo, kx, blk * kTcRows, &bar_full[st]);
          tma_load_2d(sb, &mB_hi, kb + kx, nt * BN, &bar_full[st]);
          tma_load_2d(sb + b_bytes, &mB_lo, kb + kx, nt * BN, &bar_full[st]);
          s_issued = it + 1;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = tc_idesc_bf16(kTcRows, BN);
      int it = 0;
      for (int j = j_begin; j < j_end && !s_abort; ++j) {
        int nt, blk, c0, c1, kb;
        tile(tile_of(j), nt, blk, c0, c1, kb);
        const int jj = j - j_begin, buf = jj & 1;
        const uint32_t acc = tmem + (uint32_t)buf * ncols;
        if (!mbar_wait(&bar_tempty[buf], ((uint32_t)(jj >> 1) & 1u) ^ 1u, wait_ns)) {  // accumulator free
          s_abort = 1;
          break;
        }
        tc_fence_after();
        for (int ch = c0; ch < c1; ++ch, ++it) {
          const int st = it % stages;
          const uint32_t ph = (uint32_t)(it / stages) & 1u;
          if (!mbar_wait(&bar_full[st], ph, wait_ns)) {
            s_abort = 1;
            break;
          }
          s_consumed = it + 1;
          tc_fence_after();
          const uint32_t a_hi = smem_u32(base + (size_t)st * stage_bytes);
          const uint32_t a_lo = a_hi + a_bytes, b_hi = a_hi + 2 * a_bytes, b_lo = b_hi + b_bytes;
#pragma unroll
          for (int k = 0; k < kTcK / 16; ++k) {
            const uint32_t o = 32u * k;
            tc_mma(acc, swz_desc(a_lo + o), swz_desc(b_hi + o), idesc, (ch > c0 || k > 0) ? 1u : 0u);
            tc_mma(acc, swz_desc(a_hi + o), swz_desc(b_lo + o), idesc, 1u);
            tc_mma(acc, swz_desc(a_hi + o), swz_desc(b_hi + o), idesc, 1u);
          }
          tc_commit(&bar_empty[st]);
        }
        tc_commit(&bar_tfull[buf]);  // (also with no MMAs: the epilogue then stores zeros)
      }
      tc_commit(&bar_fin);  // arrives once every MMA this CTA issued is done (aborted or not)
    }
  } else {
    // epilogue: warp w reads tensor-memory lanes 32 (w % 4) .. + 31 = tile rows
    const int q = warp & 3, ew = warp - 2;
    for (int j = j_begin; j < j_end; ++j) {
      const int t = tile_of(j);
      int nt, blk, c0, c1, kb;
      tile(t, nt, blk, c0, c1, kb);
      const int jj = j - j_begin, nk = c1 - c0, buf = jj & 1;
      const bool ok = mbar_wait(&bar_tfull[buf], (uint32_t)(jj >> 1) & 1u, wait_ns);
      tc_fence_after();
      const bool store = __all_sync(0xffffffffu, ok && !s_abort);
      if (!store) {
        s_abort = 1;
        break;
      }
      const uint32_t tacc = tmem + (uint32_t)buf * ncols + ((uint32_t)(q * 32) << 16);
      const int n0 = nt * BN, rt = blk * kTcRows + q * 32, r = rt + lane;
      for (int cc = 0; cc < BN; cc += 16) {
        float v[16];
        if (nk > 0) {
          tc_ld16(tacc + (uint32_t)cc, v);
        } else {
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) v[jj] = 0.f;
        }
        if (mode == 0) {
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) s_stage[ew][lane][jj] = v[jj];
          __syncwarp();
          float* o = out + (int64_t)(t / (ntn * blocks)) * out_stride;
          const int col = lane & 15, n = n0 + cc + col;
#pragma unroll 4
          for (int rr = 0; rr < 32; rr += 2) {
            const int row = rr + (lane >> 4);
            if (rt + row < R && n < N) o[(int64_t)(rt + row) * N + n] = scale * s_stage[ew][row][col];
          }
          __syncwarp();
        } else if (r < R) {
#pragma unroll
          for (int jj = 0; jj < 16; ++jj) {
            const int n = n0 + cc + jj;
            if (n < N) {
              const float x = scale * v[jj];
              const __nv_bfloat16 h = __float2bfloat16_rn(x);
              oh[(int64_t)n * ld + r] = h;
              ol[(int64_t)n * ld + r] = __float2bfloat16_rn(x - __bfloat162float(h));
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&bar_tempty[buf]);  // accumulator read out
    }
  }

  tc_fence_before();
  __syncthreads();
  if (s_abort && threadIdx.x == 0) {
    *err = 1.0;
    // copies in flight land, then the issued MMAs finish (the issuer's last commit)
    for (int it = s_consumed; it < s_issued; ++it)
      if (!mbar_wait(&bar_full[it % stages], (uint32_t)(it / stages) & 1u, wait_ns)) break;
    mbar_wait(&bar_fin, 0, wait_ns);
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tc_dealloc(tmem, 2 * ncols);
  }
}

// Sum of `parts` FP32 partials (R x N row-major, R*N apart) -> transposed
// split: hi[n * ld + r], lo[n * ld + r] (the first product with its K range
// split, feeding the second product's B operand).
__global__ void k_finish_t(const float* __restrict__ part, int parts, int R, int N, int64_t ld,
                           __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                           const double* __restrict__ pred) {
  if (pred != nullptr && pred[6] != 0.0) return;
  __shared__ float t[32][33];
  const int r0 = blockIdx.x * 32, n0 = blockIdx.y * 32;
  const int64_t RN = (int64_t)R * N;
  for (int rr = threadIdx.y; rr < 32; rr += blockDim.y) {
    const int r = r0 + rr, n = n0 + threadIdx.x;
    float v = 0.f;
    if (r < R && n < N)
      for (int q = 0; q < parts; ++q) v += part[q * RN + (int64_t)r * N + n];  // fixed order
    t[rr][threadIdx.x] = v;
  }
  __syncthreads();
  for (int rr = threadIdx.y; rr < 32; rr += blockDim.y) {
    const int n = n0 + rr, r = r0 + threadIdx.x;
    if (n < N && r < R) {
      const float x = t[threadIdx.x][rr];
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      hi[(int64_t)n * ld + r] = h;
      lo[(int64_t)n * ld + r] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
  }
}

// V (M x N row-major FP32) -> V^T split: hi[n * ld + i], lo[n * ld + i].
// With maxr != null V is BF's reduced-space lift of the input (260-267):
// entry (i, maxr[i]) is replaced by -rs[i].
__global__ void k_split_t(const float* __restrict__ V, int M, int N, int64_t ld, __nv_bfloat16* __restrict__ hi,
                          __nv_bfloat16* __restrict__ lo, const double* __restrict__ pred,
                          const int32_t* __restrict__ maxr = nullptr, const float* __restrict__ rs = nullptr) {
  if (pred != nullptr && pred[6] != 0.0) return;
  __shared__ float t[32][33];
  const int i0 = blockIdx.x * 32, n0 = blockIdx.y * 32;
  for (int rr = threadIdx.y; rr < 32; rr += blockDim.y) {
    const int i = i0 + rr, n = n0 + threadIdx.x;
    float v = 0.f;
    if (i < M && n < N) {
      v = V[(int64_t)i * N + n];
      if (maxr != nullptr && n == min(max(maxr[i], 0), N - 1)) v = -rs[i];
    }
    t[rr][threadIdx.x] = v;
  }
  __syncthreads();
  for (int rr = threadIdx.y; rr < 32; rr += blockDim.y) {
    const int n = n0 + rr, i = i0 + threadIdx.x;
    if (n < N && i < M) {
      const float x = t[threadIdx.x][rr];
      const __nv_bfloat16 h = __float2bfloat16_rn(x);
      hi[(int64_t)n * ld + i] = h;
      lo[(int64_t)n * ld + i] = __float2bfloat16_rn(x - __bfloat162float(h));
    }
  }
}

// Line-search probes -> the K-major split operand of their F products:
// probe b = blockIdx.z, dX = (float)(Xc[b] - X0) (M x N, FP64 in), written
// transposed as rows b * N + n of hi / lo (hi[(b * N + n) * ld + i]), so one
// tensor-core product over N' = nb * N columns gives F.dX of every probe.
__global__ void k_delta_split_t(const double* __restrict__ Xc, const double* __restrict__ X0, int M, int N,
                                int64_t ld, __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo) {
  __shared__ float t[32][33];
  const int b = blockIdx.z;
  const double* x = Xc + (int64_t)b * M * N;
  const int i0 = blockIdx.x * 32, n0 = blockIdx.y * 32;
  for (int rr = threadIdx.y; rr < 32; rr += blockDim.y) {
    const int i = i0 + rr, n = n0 + threadIdx.x;
    float v = 0.f;
    if (i < M && n < N) {
      const int64_t k = (int64_t)i * N + n;
      v = (float)(x[k] - X0[k]);
    }
    t[rr][threadIdx.x] = v;
  }
  __syncthreads();
  const int64_t row0 = (int64_t)b * N;
  for (int rr = threadIdx.y; rr < 32; rr += blockDim.y) {
    const int n = n0 + rr, i = i0 + threadIdx.x;
    if (n < N && i < M) {
      const float v = t[threadIdx.x][rr];
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      hi[(row0 + n) * ld + i] = h;
      lo[(row0 + n) * ld + i] = __float2bfloat16_rn(v - __bfloat162float(h));
    }
  }
}

// Tensor-core mixed CG, one launch before the Hessian product: the p update
// p = beta p + z (2075; skipped when do_update = 0, the first iteration),
// then V = p, or in the reduced space BF's lift (260-267) V = p with entry
// (i, maxr[i]) = -rs[i], rs[i] = sum(p(i,:)) - p(i,maxr[i]) (written to rs),
// and V's transposed split hi[n * ld + i], lo[n * ld + i] (the F.V
// product's K-major operand).  One block of 32 x Y threads owns 32 whole
// rows (thread (x, y) always handles column x of rows y, y + Y, ...): in the
// reduced space it first updates them and forms their sums (a warp tree per
// row), then transposes the lifted rows tile by tile; in the full space it
// updates and transposes in one pass.  Replaces k_cg_pupdate / k_cg_lift32
// + k_split_t.
template <int Y>
__device__ __forceinline__ void cg_lift_split_body(int bx, const double* __restrict__ sc, int do_update, int M, int N,
                                                   float* __restrict__ p, const float* __restrict__ z,
                                                   const int32_t* __restrict__ maxr, float* __restrict__ rs,
                                                   int64_t ld, __nv_bfloat16* __restrict__ hi,
                                                   __nv_bfloat16* __restrict__ lo) {
  static_assert(32 % Y == 0, "rows per thread");
  constexpr int Q = 32 / Y;
  __shared__ float t[32][33];
  __shared__ float s_rest[32];
  __shared__ int s_m[32];
  const int tx = threadIdx.x, ty = threadIdx.y;  // blockDim = (32, Y)
  const int i0 = bx * 32;
  const float beta = do_update ? (float)sc[SC_V2] : 0.f;
  const bool reduced = maxr != nullptr;
  if (reduced) {
    // pass 1: update the block's rows, sum them
    float sum[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) sum[q] = 0.f;
    for (int n0 = 0; n0 < N; n0 += 32) {
      const int n = n0 + tx;
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int i = i0 + ty + Y * q;
        if (i < M && n < N) {
          const int64_t k = (int64_t)i * N + n;
          float pv = p[k];
          if (do_update) {
            pv = fmaf(beta, pv, z[k]);
            p[k] = pv;
          }
          sum[q] += pv;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) sum[q] += __shfl_xor_sync(0xffffffffu, sum[q], o);
    __syncthreads();  // the updated rows are visible to the whole block
    if (tx == 0) {
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const int r = ty + Y * q, i = i0 + r;
        if (i < M) {
          const int m = min(max(maxr[i], 0), N - 1);
          const float rest = sum[q] - p[(int64_t)i * N + m];
          s_rest[r] = rest;
          s_m[r] = m;
          rs[i] = rest;
        }
      }
    }
    __syncthreads();
  }
  // transpose tile by tile (pass 2 in the reduced space)
  for (int n0 = 0; n0 < N; n0 += 32) {
    for (int rr = ty; rr < 32; rr += Y) {
      const int i = i0 + rr, n = n0 + tx;
      float v = 0.f;
      if (i < M && n < N) {
        const int64_t k = (int64_t)i * N + n;
        v = p[k];
        if (!reduced && do_update) {
          v = fmaf(beta, v, z[k]);
          p[k] = v;
        }
        if (reduced && n == s_m[rr]) v = -s_rest[rr];
      }
      t[rr][tx] = v;
    }
    __syncthreads();
    for (int rr = ty; rr < 32; rr += Y) {
      const int n = n0 + rr, i = i0 + tx;
      if (n < N && i < M) {
        const float x = t[tx][rr];
        const __nv_bfloat16 h = __float2bfloat16_rn(x);
        hi[(int64_t)n * ld + i] = h;
        lo[(int64_t)n * ld + i] = __float2bfloat16_rn(x - __bfloat162float(h));
      }
    }
    __syncthreads();
  }
}

template <int Y>
__global__ void __launch_bounds__(32 * Y) k_cg_lift_split(const double* __restrict__ sc, int do_update, int M, int N,
                                                          float* __restrict__ p, const float* __restrict__ z,
                                                          const int32_t* __restrict__ maxr, float* __restrict__ rs,
                                                          int64_t ld, __nv_bfloat16* __restrict__ hi,
                                                          __nv_bfloat16* __restrict__ lo) {
  if (sc != nullptr && sc[SC_DONE] != 0.0) return;
  cg_lift_split_body<Y>(blockIdx.x, sc, do_update, M, N, p, z, maxr, rs, ld, hi, lo);
}

}  // namespace pqdts
