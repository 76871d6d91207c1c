// Lockstep CG of a group of instances that share F (the resampled and
// gamma-swept members of a batch: the same probes, different P and gamma).
// One launch per CG phase serves every member of the group:
//
//   k_cg_lift_split_b   p update + BF's lift + operand split of every member,
//                       member j's V^T in rows j*N .. j*N + N-1 of one
//                       (G*N) x M operand;
//   tensor-core F.V and F^T.(2 F.V) of that operand (an N' = G*N product:
//                       the members are extra columns of one contraction);
//   k_hvp_epi32_rows_b  every member's Hessian row epilogue (its gamma, its
//                       space, its active set) from its column window of the
//                       transposed product, p.Hp into its own scalars;
//   k_cg_step32_b       every member's step, r.z and r.r and CG scalars.
//
// A member's table entry points at its own vectors and scalars; the
// per-member arithmetic is the single-instance kernels' (shared bodies).
// Members whose CG has ended (their own exit test) skip their blocks; the
// group's done flag, which predicates the tensor-core products, is set when
// the last active member's CG ends.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

namespace pqdts {

struct CGMember {
  float *p, *z, *rs, *Hp, *sn, *r;
  const float* rsq;     // 1/sqrt(bdfac * Bdiag) per row
  const int32_t* maxr;  // null: full space
  const int8_t* ik;     // active-set mask
  double* sc;           // the member's CG scalars
  double *part_rz, *part_rr, *dpart;
  unsigned *cnt_epi, *cnt_step;  // the member's grid-completion counters
  double* log;                   // the member's CG log rows
  float c2gam;                   // 2 gamma of the member
  int active;                    // 0: not part of this CG
};

struct CGGroup {
  unsigned* ndone;  // active members whose CG has ended (reset by the host before each CG)
  double* sc;       // group scalars: sc[SC_DONE] = 1 once all active members' CG ended
  int active;       // active members
};

template <int Y>
__global__ void __launch_bounds__(32 * Y) k_cg_lift_split_b(const CGMember* __restrict__ mem, int do_update, int M,
                                                            int N, int64_t ld, __nv_bfloat16* __restrict__ hi,
                                                            __nv_bfloat16* __restrict__ lo) {
  const CGMember& m = mem[blockIdx.y];
  if (!m.active || m.sc[SC_DONE] != 0.0) return;
  const int64_t off = (int64_t)blockIdx.y * N * ld;
  cg_lift_split_body<Y>(blockIdx.x, m.sc, do_update, M, N, m.p, m.z, m.maxr, m.rs, ld, hi + off, lo + off);
}

// Hraw: the group's transposed product partials, (M, G*N) row-major per
// split, member j's columns j*N .. j*N + N-1.
__global__ void __launch_bounds__(256) k_hvp_epi32_rows_b(const CGMember* __restrict__ mem,
                                                         const float* __restrict__ Hraw, int64_t hstride,
                                                         int64_t hplane, int M, int N, int RB, int parts) {
  const CGMember& m = mem[blockIdx.y];
  if (!m.active || m.sc[SC_DONE] != 0.0) return;
  hvp_epi32_rows_body(blockIdx.x, gridDim.x, Hraw + (int64_t)blockIdx.y * N, hstride, hplane, m.p, m.rs, m.maxr,
                      m.maxr ? 1 : 0, m.c2gam, m.ik, M, N, RB, m.Hp, m.dpart, parts, m.sc + SC_V2, m.cnt_epi);
}

__global__ void k_cg_step32_b(const CGMember* __restrict__ mem, CGGroup grp, int M, int N, int maxit) {
  const CGMember& m = mem[blockIdx.y];
  if (!m.active || m.sc[SC_DONE] != 0.0) return;
  const bool advanced = cg_step32_body(blockIdx.x, gridDim.x, m.sc, m.rsq, M, N, m.p, m.Hp, m.sn, m.r, m.z,
                                       m.part_rz, m.part_rr, m.log, maxit, m.cnt_step);
  if (advanced && threadIdx.x == 0 && m.sc[SC_DONE] != 0.0) {
    __threadfence();
    if (atomicAdd(grp.ndone, 1u) == (unsigned)grp.active - 1) grp.sc[SC_DONE] = 1.0;
  }
}

}  // namespace pqdts
