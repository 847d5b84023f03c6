// Block-band triangular sweeps on the tensor cores with the window operand in
// tensor memory.
//
// The sweep is the one described in bddc_tc.cuh: for every system and every
// 128-column tile of its right-hand side B (row-major FP32), block row k is
//     B[k] = P_k  x  [window blocks of B]
// with the precomputed panel P_k (forward: [-Linv_kk L_kj ... | Linv_kk],
// backward: [Linv_kk^T | -Linv_kk^T L_ik^T ...]).  It replaces the interior
// and preconditioner solves of MUMPS (dd_prepare_schur / dd_prepare_aug /
// dd_solve_aug, module_dd.f90:4175-4295, 5211-5486, 5843-5932).
//
// The window (M = 128 columns of B by K) is the MMA's A operand and lives in
// tensor memory: each of the 128 staging threads owns one column of the tile,
// which is one TMEM lane, and writes the TF32 hi and lo parts of its column
// there (tcgen05.st), so the MMAs read only the 64-row panel (the B operand,
// 16 KB per 32-wide K chunk, moved by cp.async.bulk) from shared memory.
// The two freshest window blocks never go through global memory on the
// critical path: the epilogue threads read a finished block row from the TMEM
// accumulator, store it as the result and split it straight into the stages
// of the two following steps that read it.  The other window blocks (older
// solved blocks and the right-hand-side block) do not depend on the previous
// steps, so the staging threads load them from global memory ahead of time,
// and the issue order (below) lets the tensor core work on them while the
// epilogue of the previous step runs.
//
// Roles (352 threads, one CTA per SM):
//   warps 0-3 and 4-7: two staging groups (each one thread per TMEM lane);
//       group (jb & 1) stages every chunk of window block jb and writes the
//       results of block jb (the epilogue), so a thread only ever reads back
//       rows of its own column that it wrote itself;
//   warp 8 (one thread): panel chunks into a ring of shared-memory slots;
//   warp 9 (one thread): the MMAs, into one of three TMEM accumulators;
//   warp 10 (one thread): follows the MMA completions chunk by chunk (one phase of
//       one stage barrier at a time) and publishes their count, which the
//       staging threads wait on before they refill a stage.  The epilogue
//       fills stages out of chunk order, and a parity wait on a barrier that
//       is two phases behind would pass early; a count cannot.
// Precision: 3xTF32 (a_lo p_hi + a_hi p_lo + a_hi p_hi, FP32 accumulation),
// or one TF32 product for a correction that is itself tiny (PASSES = 1).
//
// Every wait is bounded (limit g_tc_wait_limit, polled together with the
// CTA's abort flag).  A wait that runs out sets the abort flag; the CTA then
// waits (bounded by the full limit) for its bulk copies and MMAs in flight,
// records DE_TIMEOUT in the error word, frees its tensor memory and returns.
#pragma once

#include "bddc_batch_tc.cuh"
#include "bddc_tc.cuh"

namespace bddc {

constexpr int SWT_AST = 5;                       // TMEM stages of split window chunks
constexpr int SWT_NACC = 3;                      // TMEM accumulators (steps t, t + 1, t + 2)
constexpr int SWT_PST = 6;                       // shared-memory slots of panel chunks
constexpr int SWT_GROUP = 128;                   // threads of one staging group
constexpr int SWT_PRODUCER = 8, SWT_ISSUER = 9, SWT_TRACKER = 10;  // warps
constexpr int SWT_THREADS = 352;
constexpr uint32_t SWT_ACOL = SWT_NACC * TC_N;  // TMEM column of stage 0, after the accumulators
constexpr uint32_t SWT_TCOLS = 512;
static_assert(SWT_ACOL + SWT_AST * 2 * TC_KC <= SWT_TCOLS, "tensor memory columns");
constexpr size_t swt_smem_bytes() { return (size_t)SWT_PST * TC_PCHUNK * sizeof(float) + 128; }


// release store / acquire load of a shared-memory counter
__device__ __forceinline__ void smem_store_release(unsigned* p, unsigned v) {
  asm volatile("st.release.cta.shared::cta.u32 [%0], %1;" ::"r"(smem_u32(p)), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned smem_load_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.cta.shared::cta.u32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
  return v;
}

// bounded wait that also gives up when another thread of the CTA has aborted
__device__ __forceinline__ bool swt_wait(uint64_t* bar, uint32_t parity, long long limit,
                                         const volatile int* abort_flag) {
  for (long long i = 0; i < limit; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63) == 63 && *abort_flag) return false;
  }
  return false;
}

// Window of sweep step t (block row k): the blocks of "age" a = 0 .. nblk - 1,
// age 0 being block k itself (the right-hand side) and age a the block solved
// a steps earlier (forward k - a, backward k + a); the panel holds block jb at
// position jb - j0.  Forward sweeps of identity columns start at row s0 and
// skip the zero blocks above it.
struct SwWin {
  int k, j0, nblk;
};

__device__ __forceinline__ SwWin sw_win(int dir, int nb, int w, int s0, int k) {
  SwWin r;
  r.k = k;
  if (dir == 0) {
    r.j0 = k - min(k, w);
    r.nblk = k - max(r.j0, s0) + 1;
  } else {
    r.j0 = k;
    r.nblk = min(w, nb - 1 - k) + 1;
  }
  return r;
}

// Bounded wait until the counter reaches `target`.
__device__ __forceinline__ bool swt_wait_count(const unsigned* counter, unsigned target, long long limit,
                                               const volatile int* abort_flag) {
  for (long long i = 0; i < limit; ++i) {
    if (smem_load_acquire(counter) >= target) return true;
    if ((i & 63) == 63 && *abort_flag) return false;
    __nanosleep(20);  // back off: spinning warps take issue slots from the working ones
  }
  return false;
}

// Issue order.  The chunks of step t (two 32-row halves per window block) fall
// into three parts: A(t) = the blocks of age >= 3 and the right-hand side
// (read from global memory), B(t) = the block of age 2 and C(t) = the block
// of age 1 (both handed over by the epilogue of the step that made them).
// "Macro step" t issues A(t), C(t - 1), B(t), so the MMAs of A(t) and B(t)
// run while the epilogue of step t - 1 (which needs C(t - 1) complete) moves
// that step's results out; the epilogue of step t - 2 supplies C(t - 1) and
// B(t), which are adjacent in the order.  Steps use accumulators t mod 3.
__device__ __forceinline__ int sw_nA(const SwWin& W) { return 2 * (1 + max(0, W.nblk - 3)); }
__device__ __forceinline__ int sw_nB(const SwWin& W) { return W.nblk >= 3 ? 2 : 0; }
__device__ __forceinline__ int sw_nC(const SwWin& W) { return W.nblk >= 2 ? 2 : 0; }

// block of age a
__device__ __forceinline__ int sw_block(int dir, const SwWin& W, int a) { return dir == 0 ? W.k - a : W.k + a; }

// chunk q of part A: the oldest blocks first, the right-hand side last
__device__ __forceinline__ int sw_A_block(int dir, const SwWin& W, int q) {
  const int p = q >> 1, nold = max(0, W.nblk - 3);
  return sw_block(dir, W, p < nold ? W.nblk - 1 - p : 0);
}

__device__ __forceinline__ int sw_pq(const SwWin& W, int jb, int half) { return 2 * (jb - W.j0) + half; }

template <int PASSES, bool ACC>
__global__ void __launch_bounds__(SWT_THREADS, 1)
    k_band_sweep_tm(const TcDesc* __restrict__ td, const float* __restrict__ ppool, float* __restrict__ bpool,
                    int dir, int* __restrict__ err, int* __restrict__ maxabs) {
  const TcDesc d = td[blockIdx.y];
  const int c0 = blockIdx.x * TC_M;
  if (c0 >= d.ncol || d.nb == 0) return;
  const int ld = d.ncol;
  float* B = bpool + d.oB;
  const float* P = ppool + (dir == 0 ? d.oPf : d.oPb);
  const uint32_t pbytes = (PASSES == 1 ? TC_PCHUNK / 2 : TC_PCHUNK) * 4;  // hi half first in a chunk
  // a forward sweep of a tile inside the identity columns (pad = their
  // count) starts at the tile's diagonal block row: the rows above stay zero
  const int s0 = (dir == 0 && c0 + TC_M <= d.pad) ? c0 / NB : 0;
  const int nsteps = d.nb - s0;
  auto row_of = [&](int t) { return dir == 0 ? s0 + t : d.nb - 1 - t; };
  auto win = [&](int t) { return sw_win(dir, d.nb, d.w, s0, row_of(t)); };
  const long long limit = g_tc_wait_limit;

  extern __shared__ __align__(128) unsigned char swt_raw[];
  float* sP = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(swt_raw) + 127) & ~uintptr_t(127));
  __shared__ __align__(8) uint64_t bar_afull[SWT_AST], bar_aempty[SWT_AST];
  __shared__ __align__(8) uint64_t bar_pfull[SWT_PST], bar_pfree[SWT_PST];
  __shared__ __align__(8) uint64_t bar_accfull[SWT_NACC], bar_tfree[SWT_NACC];
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  __shared__ long long last_pload[SWT_PST], last_mma;
  __shared__ unsigned mma_done;  // chunks whose MMAs have completed, in order

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < SWT_AST; ++s) {
      mbar_init(&bar_afull[s], SWT_GROUP);
      mbar_init(&bar_aempty[s], 1);
    }
    for (int s = 0; s < SWT_PST; ++s) {
      mbar_init(&bar_pfull[s], 1);
      mbar_init(&bar_pfree[s], 1);
      last_pload[s] = -1;
    }
    for (int b = 0; b < SWT_NACC; ++b) {
      mbar_init(&bar_accfull[b], 1);
      mbar_init(&bar_tfree[b], SWT_GROUP);
    }
    abort_flag = 0;
    last_mma = -1;
    mma_done = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(SWT_TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  // total number of chunks in the issue order
  auto total_chunks = [&]() -> long long {
    long long n = 0;
    for (int t = 0; t < nsteps; ++t) {
      const SwWin W = win(t);
      n += sw_nA(W) + sw_nB(W) + sw_nC(W);
    }
    return n;
  };

  if (warp == SWT_TRACKER) {
    // ------------------------------------------------ MMA completion tracker (one thread)
    if (lane == 0) {
      const long long n = total_chunks();
      for (long long g = 0; g < n; ++g) {
        if (!swt_wait(&bar_aempty[g % SWT_AST], (uint32_t)((g / SWT_AST) & 1), limit, &abort_flag)) {
          abort_flag = 1;
          break;
        }
        smem_store_release(&mma_done, (unsigned)(g + 1));
      }
    }
  } else if (warp == SWT_PRODUCER || warp == SWT_ISSUER) {
    if (lane == 0) {
      const bool producer = warp == SWT_PRODUCER;
      constexpr uint32_t idesc = tc_idesc(TC_M, TC_N);
      long long g = 0;
      bool ok = true;
      // one chunk of step t: panel chunk pq; first / last chunk of the step
      auto chunk = [&](int t, int pq, bool first, bool last) -> bool {
        if (producer) {
          const int s = (int)(g % SWT_PST);
          const long long use = g / SWT_PST;
          if (abort_flag || (use > 0 && !swt_wait(&bar_pfree[s], (uint32_t)((use - 1) & 1), limit, &abort_flag)))
            return false;
          mbar_expect_tx(&bar_pfull[s], pbytes);
          bulk_g2s(sP + s * TC_PCHUNK, P + panel_chunk(0, d.w, row_of(t), pq), pbytes, &bar_pfull[s]);
          last_pload[s] = g;
        } else {
          const int b = t % SWT_NACC;
          if (first && t >= SWT_NACC &&
              !swt_wait(&bar_tfree[b], (uint32_t)(((t - SWT_NACC) / SWT_NACC) & 1), limit, &abort_flag))
            return false;
          const int sa = (int)(g % SWT_AST), sp = (int)(g % SWT_PST);
          if (!swt_wait(&bar_afull[sa], (uint32_t)((g / SWT_AST) & 1), limit, &abort_flag) ||
              !swt_wait(&bar_pfull[sp], (uint32_t)((g / SWT_PST) & 1), limit, &abort_flag))
            return false;
          tc_fence_after();
          const uint32_t dacc = tmem + (uint32_t)(b * TC_N);
          const uint32_t a_hi = tmem + SWT_ACOL + (uint32_t)(sa * 2 * TC_KC), a_lo = a_hi + TC_KC;
          const uint32_t p_hi = smem_u32(sP + sp * TC_PCHUNK), p_lo = p_hi + TC_N * TC_KC * 4;
#pragma unroll
          for (int kk = 0; kk < TC_KC / 8; ++kk) {
            const uint32_t koff = kk * 2 * TC_LBO;
            const uint32_t acc = (!first || kk > 0) ? 1u : 0u;
            if (PASSES == 1) {
              mma_tf32_ta(dacc, a_hi + kk * 8, tc_desc(p_hi + koff), idesc, acc);
            } else {
              mma_tf32_ta(dacc, a_lo + kk * 8, tc_desc(p_hi + koff), idesc, acc);
              mma_tf32_ta(dacc, a_hi + kk * 8, tc_desc(p_lo + koff), idesc, 1u);
              mma_tf32_ta(dacc, a_hi + kk * 8, tc_desc(p_hi + koff), idesc, 1u);
            }
          }
          mma_commit(&bar_aempty[sa]);
          mma_commit(&bar_pfree[sp]);
          if (last) mma_commit(&bar_accfull[b]);
          last_mma = g;
        }
        ++g;
        return true;
      };
      for (int t = 0; t <= nsteps && ok; ++t) {
        if (t < nsteps) {  // A(t)
          const SwWin W = win(t);
          const int n = sw_nA(W);
          for (int q = 0; q < n && ok; ++q)
            ok = chunk(t, sw_pq(W, sw_A_block(dir, W, q), q & 1), q == 0, W.nblk == 1 && q == n - 1);
        }
        if (t >= 1 && ok) {  // C(t - 1): the last chunks of step t - 1
          const SwWin W = win(t - 1);
          const int jb = sw_block(dir, W, 1);
          for (int q = 0; q < sw_nC(W) && ok; ++q) ok = chunk(t - 1, sw_pq(W, jb, q), false, q == 1);
        }
        if (t < nsteps && ok) {  // B(t)
          const SwWin W = win(t);
          const int jb = sw_block(dir, W, 2);
          for (int q = 0; q < sw_nB(W) && ok; ++q) ok = chunk(t, sw_pq(W, jb, q), false, false);
        }
      }
      if (!ok) abort_flag = 1;
    }
  } else {
    // ------------------------------------------------ staging groups and epilogue
    const int G = warp >> 2;              // owns the window blocks jb with (jb & 1) == G
    const int r = tid & (SWT_GROUP - 1);  // column of the tile = TMEM lane
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    float* col = B + c0 + r;
    float* col_acc = (ACC && dir == 1 && d.oAcc >= 0) ? bpool + d.oAcc + c0 + r : nullptr;

    // split one 32-row piece of this thread's column into the stage of chunk g
    auto fill = [&](long long g, const float (&v)[TC_KC]) -> bool {
      const int sa = (int)(g % SWT_AST);
      // the stage's previous chunk (g - SWT_AST) must be consumed
      bool good = !abort_flag && (g < SWT_AST || swt_wait_count(&mma_done, (unsigned)(g - SWT_AST + 1), limit,
                                                                &abort_flag));
      good = __all_sync(0xffffffffu, good);  // the TMEM stores below are warp-collective
      if (!good) return false;
      tc_fence_after();
      const uint32_t ta = tmem + lane_base + SWT_ACOL + (uint32_t)(sa * 2 * TC_KC);
      float h[TC_KC];
#pragma unroll
      for (int i = 0; i < TC_KC; ++i) h[i] = tf32_rna(v[i]);
      tmem_st32(ta, h);
      if (PASSES != 1) {
#pragma unroll
        for (int i = 0; i < TC_KC; ++i) h[i] = tf32_rna(v[i] - tf32_rna(v[i]));
        tmem_st32(ta + TC_KC, h);
      }
      tmem_st_wait();
      tc_fence_before();
      mbar_arrive(&bar_afull[sa]);
      return true;
    };
    // results of step e (block row k) from its accumulator to B; each half
    // also fills chunk gC + h of part C(e + 1) and chunk gB + h of part B(e + 2)
    // when those are >= 0
    auto epilogue = [&](int e, long long gC, long long gB) -> bool {
      const int k = row_of(e), b = e % SWT_NACC;
      bool good = !abort_flag && swt_wait(&bar_accfull[b], (uint32_t)((e / SWT_NACC) & 1), limit, &abort_flag);
      good = __all_sync(0xffffffffu, good);  // the TMEM loads below are warp-collective
      if (!good) return false;
      tc_fence_after();
      // the row stride is made opaque so that the row offsets are formed here
      // rather than kept live in registers across the sweep
      long long lds = ld;
      asm volatile("" : "+l"(lds));
#pragma unroll 1
      for (int h = 0; h < 2; ++h) {
        float v[TC_KC];
        {
          float v0[16], v1[16];
          tmem_ld16(tmem + lane_base + (uint32_t)(b * TC_N + h * TC_KC), v0);
          tmem_ld16(tmem + lane_base + (uint32_t)(b * TC_N + h * TC_KC + 16), v1);
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            v[i] = v0[i];
            v[16 + i] = v1[i];
          }
        }
        if (h == 1) {  // both halves are in registers: the accumulator may take step e + 3
          tc_fence_before();
          mbar_arrive(&bar_tfree[b]);
        }
        float* dst = col + (long long)(k * NB + h * TC_KC) * lds;
#pragma unroll
        for (int i = 0; i < TC_KC; ++i) dst[(long long)i * lds] = v[i];
        if (maxabs) {  // largest |result| of the system (non-negative FP32 bits order like integers)
          float m = 0.f;
#pragma unroll
          for (int i = 0; i < TC_KC; ++i) m = fmaxf(m, fabsf(v[i]));
          for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
          if (lane == 0) atomicMax(maxabs + blockIdx.y, __float_as_int(m));
        }
        if (ACC && col_acc) {
          float* dst2 = col_acc + (long long)(k * NB + h * TC_KC) * lds;
          float a[TC_KC];
#pragma unroll
          for (int i = 0; i < TC_KC; ++i) a[i] = dst2[(long long)i * lds];
#pragma unroll
          for (int i = 0; i < TC_KC; ++i) dst2[(long long)i * lds] = a[i] + v[i];
        }
        if (gC >= 0 && !fill(gC + h, v)) return false;
        if (gB >= 0 && !fill(gB + h, v)) return false;
      }
      return true;
    };
    auto load = [&](int jb, int half, float (&v)[TC_KC]) {
      const float* src = col + (long long)(jb * NB + half * TC_KC) * ld;
#pragma unroll
      for (int i = 0; i < TC_KC; ++i) v[i] = src[(long long)i * ld];
    };
    // The next chunk of this group after position (t, part A, chunk q): true
    // with its block, half and sequence number when it is a chunk of part A
    // (read from global memory); false when the group's next event is an
    // epilogue (whose chunks it makes itself) or the sequence ends.  Every
    // block that a part-A chunk reads was written by this group's own
    // epilogue earlier in the order, so a prefetch never reads stale rows.
    auto next_load = [&](int t, int q, long long g, int& njb, int& nhalf, long long& ng) -> bool {
      ng = g + 1;
      int qq = q + 1;
      for (int tt = t; tt < nsteps; ++tt) {
        const SwWin W = win(tt);
        for (; qq < sw_nA(W); ++qq, ++ng) {
          const int jb = sw_A_block(dir, W, qq);
          if ((jb & 1) == G) {
            njb = jb;
            nhalf = qq & 1;
            return true;
          }
        }
        // then part C(tt - 1), where the epilogue of step tt - 2 runs, and part B(tt)
        if (tt >= 2 && (row_of(tt - 2) & 1) == G) return false;
        if (tt >= 1) ng += sw_nC(win(tt - 1));
        ng += sw_nB(W);
        qq = 0;
      }
      return false;
    };

    float vn[TC_KC];
    long long gn = -1;  // sequence number of the chunk held in vn
    long long g = 0;
    bool ok = true;
    for (int t = 0; t <= nsteps && ok; ++t) {
      if (t < nsteps) {  // A(t)
        const SwWin W = win(t);
        const int n = sw_nA(W);
        for (int q = 0; q < n; ++q, ++g) {
          const int jb = sw_A_block(dir, W, q);
          if ((jb & 1) != G) continue;
          float v[TC_KC];
          if (gn == g) {
#pragma unroll
            for (int i = 0; i < TC_KC; ++i) v[i] = vn[i];
          } else {
            load(jb, q & 1, v);
          }
          {
            int njb, nhalf;
            long long ng;
            gn = -1;
            if (next_load(t, q, g, njb, nhalf, ng)) {
              load(njb, nhalf, vn);
              gn = ng;
            }
          }
          if (!fill(g, v)) {
            ok = false;
            break;
          }
        }
        if (!ok) break;
      }
      long long gC = -1, gB = -1;
      int nC = 0;
      if (t >= 1) {  // C(t - 1)
        nC = sw_nC(win(t - 1));
        if (nC) gC = g;
        g += nC;
      }
      if (t < nsteps) {  // B(t)
        const int nB = sw_nB(win(t));
        if (nB) gB = g;
        g += nB;
      }
      // the epilogue of step t - 2 supplies C(t - 1) and B(t)
      if (t >= 2 && (row_of(t - 2) & 1) == G && !epilogue(t - 2, gC, gB)) ok = false;
    }
    // the last step's results: written by the group that owns its block row
    if (ok && nsteps >= 1 && (row_of(nsteps - 1) & 1) == G && !epilogue(nsteps - 1, -1, -1)) ok = false;
    if (!ok) abort_flag = 1;
  }
  // wind-down: after an abort, wait (bounded) for the copies and MMAs in flight before freeing TMEM
  __syncthreads();
  if (tid == 0 && abort_flag) {
    for (int s = 0; s < SWT_PST; ++s)
      if (last_pload[s] >= 0) mbar_wait(&bar_pfull[s], (uint32_t)((last_pload[s] / SWT_PST) & 1));
    // the MMA completions not seen yet, one phase at a time (in order, so no
    // parity wait can pass early)
    for (long long g = mma_done; g <= last_mma; ++g)
      if (!mbar_wait(&bar_aempty[g % SWT_AST], (uint32_t)((g / SWT_AST) & 1))) break;
    atomicOr(err, DE_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(SWT_TCOLS));
}

}  // namespace bddc
