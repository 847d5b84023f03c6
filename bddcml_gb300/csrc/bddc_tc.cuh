// 5th-generation tensor-core path (tcgen05, TMEM, bulk TMA) for the block-band
// triangular sweeps of the subdomain solves.
//
// One sweep step computes, for every subdomain and every 128-column tile of
// the right-hand-side block B (row-major, FP32):
//     B[k-block rows, tile] = P_k  x  B[window rows, tile]
// where the window is the band of block rows that block row k depends on and
// P_k (64 x window) is a precomputed panel with the inverted diagonal block
// folded in:
//     forward : P_k = [-Linv_kk L_k,j0 ... -Linv_kk L_k,k-1 | Linv_kk]
//     backward: Q_k = [Linv_kk^T | -Linv_kk^T L_k+1,k^T ... -Linv_kk^T L_k+w,k^T]
// so that each step is one contraction on the tensor cores.
//
// Precision: 3xTF32 (Ootomo & Yokota's split a = hi + lo with hi = tf32(a);
// a*b ~ hi*hi + hi*lo + lo*hi), FP32 accumulation in TMEM.  This is the
// FP32-class inner solve of the refinement loop in the setup.
//
// MMA shape: M = 128 (columns of B), N = 64 (rows of the output block),
// K = 8 per instruction, both operands K-major in the canonical no-swizzle
// layout (core matrices of 8 rows x 16 bytes).  The panel operand is stored
// in global memory already split and laid out per 32-wide K chunk and is
// moved by cp.async.bulk; the window operand is read from global memory,
// split into hi/lo and written into the canonical layout by all threads.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "bddc_kernels.cuh"

namespace bddc {

constexpr int TC_M = 128;            // columns of B per CTA (MMA M)
constexpr int TC_N = 64;             // output rows (MMA N)
constexpr int TC_KC = 32;            // K chunk staged per pipeline stage
constexpr int TC_THREADS = 128;
constexpr int TC_STAGES = 2;             // window stages of the sweep
constexpr int TC_PST = 3;                // panel stages of the sweep (copies two chunks ahead)
constexpr int TC_PCHUNK = TC_N * TC_KC * 2;     // floats per panel chunk (hi + lo)
constexpr int TC_ACHUNK = TC_M * TC_KC;         // floats per window-operand half (hi or lo)
constexpr uint32_t TC_LBO = 128;                // bytes between K-adjacent core matrices
constexpr uint32_t TC_SBO = (TC_KC / 4) * 128;  // bytes between 8-row groups
constexpr long long TC_SPIN_LIMIT = 1LL << 26;  // bounded waits
enum { DE_TIMEOUT = 8 };

// offset (floats) of element (row r, k) inside one canonical K-major operand
// tile of TC_KC columns
__host__ __device__ __forceinline__ int canon_off(int r, int k) {
  return (r >> 3) * (TC_SBO / 4) + (k >> 2) * (TC_LBO / 4) + (r & 7) * 4 + (k & 3);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait: returns false after the spin limit
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = TC_SPIN_LIMIT) {
  for (long long i = 0; i < limit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Spin limit of the sweeps' waits (their wind-down waits use TC_SPIN_LIMIT).
// Settable for tests of the timeout path (bddcml_set_wait_limit_c).
static __device__ long long g_tc_wait_limit = TC_SPIN_LIMIT;

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: canonical K-major, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((TC_LBO >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((TC_SBO >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of the 5th-generation tensor core
  return d;
}

// instruction descriptor: kind::tf32, D = F32, A = B = TF32, both K-major
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

struct TcDesc {
  int nb, w, ncol;
  int pad;           // leading identity columns of B (forward sweeps skip the zero rows above them)
  long long oB;      // RHS block (row-major, ld = ncol) in the work pool
  long long oPf;     // forward panels in the panel pool
  long long oPb;     // backward panels
  long long oAcc;    // < 0, or a block (same shape as B) the backward sweep adds its result into
  int lower = 0;     // 1: the result is a symmetric matrix's inverse on the identity columns, of which
                     // only the lower triangle is wanted: backward sweeps of a tile inside them stop
                     // at the tile's diagonal block row
};

// panel storage: block row k, chunk q at ((k * (w+1)*2) + q) * TC_PCHUNK
__host__ __device__ __forceinline__ long long panel_chunk(long long base, int w, int k, int q) {
  return base + ((long long)k * (w + 1) * 2 + q) * TC_PCHUNK;
}

// Complete forward (dir = 0) or backward (dir = 1) sweep: one CTA owns one
// 128-column tile of one system's right-hand side and walks all block rows;
// tiles are independent, so no grid-wide synchronisation is needed and the
// band window of a tile (w+1 block rows x 128 columns) stays in L2 between
// consecutive block rows.  grid (max column tiles, batch).
//
// Warp roles: warps 0-3 (one thread per column of the tile) stage the window
// chunks (global -> registers -> TF32 split -> canonical shared layout) and
// move finished block rows from TMEM to global memory; lane 0 of warp 4
// issues the panel copies (cp.async.bulk) and the MMAs.  Stages are handed
// over with mbarriers, so the staging warps run ahead of the tensor core.
// Two TMEM accumulators alternate between block rows; the block row finished
// last (the only part of a window that depends on the previous step) is
// placed at the end of the next window, and the previous row's results are
// written out after the first chunks of the next row are queued.
//
// passes = 3: 3xTF32 (FP32-class result); passes = 1: one TF32 product
// (hi x hi, relative error ~1e-3), for a refinement correction that is
// itself ~1e-10 of the solution.  With oAcc >= 0 the backward sweep also
// adds each finished block row into the block at oAcc.
constexpr int SW_THREADS = TC_THREADS + 32;

struct SweepChunk {
  int jb;    // block row of B read by this chunk
  int pq;    // panel chunk index (2 * block position in the panel + half)
  int half;  // which 32-row half of the block
  bool dep;  // reads the block row finished by the previous step
};

// q-th chunk of the window of block row k (the freshest block last)
__device__ __forceinline__ SweepChunk sweep_chunk(int dir, int nb, int w, int k, int q) {
  int j0, nblk;
  if (dir == 0) { j0 = k - min(k, w); nblk = k - j0 + 1; }
  else { j0 = k; nblk = min(w, nb - 1 - k) + 1; }
  const int p = q >> 1;
  SweepChunk c;
  c.half = q & 1;
  c.dep = false;
  if (nblk == 1) {
    c.jb = k;
  } else if (p == nblk - 1) {
    c.jb = dir == 0 ? k - 1 : k + 1;
    c.dep = true;
  } else if (dir == 0) {
    c.jb = p < nblk - 2 ? j0 + p : k;
  } else {
    c.jb = p == 0 ? k : k + 1 + p;
  }
  c.pq = 2 * (c.jb - j0) + c.half;
  return c;
}

__device__ __forceinline__ int sweep_nchunk(int dir, int nb, int w, int k) {
  return 2 * (dir == 0 ? min(k, w) + 1 : min(w, nb - 1 - k) + 1);
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// ACC: 0 none; 1 the backward sweep adds its result into the block at oAcc;
// 2 likewise, into the FP32 pair (block at oAcc - one component, block at
// oAcc) kept renormalised
template <int PASSES, int ACC>
__global__ void __launch_bounds__(SW_THREADS, 2)
    k_band_sweep_tc(const TcDesc* __restrict__ td, const float* __restrict__ ppool, float* __restrict__ bpool,
                    int dir, int* __restrict__ err, int* __restrict__ maxabs) {
  constexpr int passes = PASSES;
  const TcDesc d = td[blockIdx.y];
  const long long limit = g_tc_wait_limit;
  const int c0 = blockIdx.x * TC_M;
  if (c0 >= d.ncol || d.nb == 0) return;
  const int ld = d.ncol;
  float* B = bpool + d.oB;
  const float* P = ppool + (dir == 0 ? d.oPf : d.oPb);
  const uint32_t pbytes = (passes == 1 ? TC_PCHUNK / 2 : TC_PCHUNK) * 4;  // hi half first in a chunk

  extern __shared__ __align__(128) unsigned char sw_smem[];
  float* sA = reinterpret_cast<float*>(sw_smem);                // [stage][hi|lo][TC_ACHUNK]
  float* sP = sA + TC_STAGES * 2 * TC_ACHUNK;                    // [panel stage][TC_PCHUNK]
  __shared__ __align__(8) uint64_t bar_a[TC_STAGES], bar_mma[TC_STAGES], bar_acc[2], bar_tfree[2];
  __shared__ __align__(8) uint64_t bar_p[TC_PST], bar_pfree[TC_PST];
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  __shared__ long long last_commit, tma_pending[TC_PST];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // a forward sweep of a tile inside the identity columns (pad = their
  // count) starts at the tile's diagonal block row: the rows above stay zero
  const int s0 = (dir == 0 && c0 + TC_M <= d.pad) ? c0 / NB : 0;
  // with `lower`, the backward sweep of such a tile stops at its diagonal block
  // row: the rows above hold the upper triangle, which the caller does not read
  const int s1 = (dir == 1 && d.lower && c0 + TC_M <= d.pad) ? c0 / NB : 0;
  const int nsteps = d.nb - s0 - s1;
  auto row_of = [&](int sidx) { return dir == 0 ? s0 + sidx : d.nb - 1 - sidx; };
  if (tid == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(&bar_a[s], TC_THREADS);
      mbar_init(&bar_mma[s], 1);
    }
    for (int s = 0; s < TC_PST; ++s) {
      mbar_init(&bar_p[s], 1);
      mbar_init(&bar_pfree[s], 1);
      tma_pending[s] = -1;
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&bar_acc[b], 1);
      mbar_init(&bar_tfree[b], TC_THREADS);
    }
    abort_flag = 0;
    last_commit = -1;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(2 * TC_N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (warp == TC_THREADS / 32) {
    // ------------------------------------------------ issuer (one thread)
    if (lane == 0) {
      constexpr uint32_t idesc = tc_idesc(TC_M, TC_N);
      auto issue_panel = [&](int st, int k, int pq, long long gg) {
        mbar_expect_tx(&bar_p[st], pbytes);
        bulk_g2s(sP + st * TC_PCHUNK, P + panel_chunk(0, d.w, k, pq), pbytes, &bar_p[st]);
        tma_pending[st] = gg;
      };
      // panel copies run TC_PST - 1 chunks ahead of the MMAs (cursor ps, pqi)
      int ps = 0, pqi = 0;
      long long gp = 0;
      auto prefetch = [&]() -> bool {
        if (ps >= nsteps) return true;
        const int pst = (int)(gp % TC_PST);
        if (gp >= TC_PST && !mbar_wait(&bar_pfree[pst], (uint32_t)(((gp - TC_PST) / TC_PST) & 1), limit)) return false;
        const int kp = row_of(ps);
        issue_panel(pst, kp, sweep_chunk(dir, d.nb, d.w, kp, pqi).pq, gp);
        ++gp;
        if (++pqi == sweep_nchunk(dir, d.nb, d.w, kp)) { pqi = 0; ++ps; }
        return true;
      };
      for (int i = 0; i < TC_PST - 1; ++i) prefetch();
      long long g = 0;
      for (int sidx = 0; sidx < nsteps && !abort_flag; ++sidx) {
        const int k = row_of(sidx), b = sidx & 1;
        const int nchunk = sweep_nchunk(dir, d.nb, d.w, k);
        const uint32_t dacc = tmem + (uint32_t)(b * TC_N);
        if (sidx >= 2 && !mbar_wait(&bar_tfree[b], (uint32_t)(((sidx - 2) >> 1) & 1), limit)) { abort_flag = 1; break; }
        for (int q = 0; q < nchunk; ++q, ++g) {
          const int st = (int)(g % TC_STAGES), pst = (int)(g % TC_PST);
          if (!mbar_wait(&bar_a[st], (uint32_t)((g / TC_STAGES) & 1), limit) ||
              !mbar_wait(&bar_p[pst], (uint32_t)((g / TC_PST) & 1), limit)) { abort_flag = 1; break; }
          tma_pending[pst] = -1;
          tc_fence_after();
          const uint32_t a_hi = smem_u32(sA + (st * 2 + 0) * TC_ACHUNK);
          const uint32_t a_lo = smem_u32(sA + (st * 2 + 1) * TC_ACHUNK);
          const uint32_t p_hi = smem_u32(sP + pst * TC_PCHUNK);
          const uint32_t p_lo = p_hi + TC_N * TC_KC * 4;
          if (passes == 1) {
#pragma unroll
            for (int kk = 0; kk < TC_KC / 8; ++kk) {
              const uint32_t koff = kk * 2 * TC_LBO;
              mma_tf32(dacc, tc_desc(a_hi + koff), tc_desc(p_hi + koff), idesc, (q > 0 || kk > 0) ? 1u : 0u);
            }
          } else {
#pragma unroll
            for (int kk = 0; kk < TC_KC / 8; ++kk) {
              const uint32_t koff = kk * 2 * TC_LBO;
              const uint32_t acc = (q > 0 || kk > 0) ? 1u : 0u;
              mma_tf32(dacc, tc_desc(a_lo + koff), tc_desc(p_hi + koff), idesc, acc);
              mma_tf32(dacc, tc_desc(a_hi + koff), tc_desc(p_lo + koff), idesc, 1u);
              mma_tf32(dacc, tc_desc(a_hi + koff), tc_desc(p_hi + koff), idesc, 1u);
            }
          }
          mma_commit(&bar_mma[st]);
          mma_commit(&bar_pfree[pst]);
          if (q == nchunk - 1) mma_commit(&bar_acc[b]);
          last_commit = g;
          // the panel TC_PST - 1 chunks ahead, once the stage it goes to is free
          if (!prefetch()) { abort_flag = 1; break; }
        }
      }
    }
  } else {
    // ------------------------------------------------ staging + epilogue (128 threads)
    const uint32_t trow = (uint32_t)(warp * 32) << 16;
    auto load_chunk = [&](int jb, int half, float (&r)[TC_KC]) {
      const float* src = B + (long long)(jb * NB + half * TC_KC) * ld + c0 + tid;
#pragma unroll
      for (int t = 0; t < TC_KC; ++t) r[t] = src[(long long)t * ld];
    };
    // move block row `sr` from its TMEM buffer to global memory
    auto epilogue = [&](int sr) -> bool {
      const int k = row_of(sr), b = sr & 1;
      // the row stride is made opaque so that the 64 row offsets are formed
      // here rather than kept live in registers across the sweep
      long long lds = ld;
      asm volatile("" : "+l"(lds));
      float* dst = B + (long long)(k * NB) * lds + c0 + tid;
      float* dst2 = (ACC && dir == 1 && d.oAcc >= 0) ? bpool + d.oAcc + (long long)(k * NB) * lds + c0 + tid : nullptr;
      if (!mbar_wait(&bar_acc[b], (uint32_t)((sr >> 1) & 1), limit)) { abort_flag = 1; return false; }
      tc_fence_after();
      float vmax = 0.f;
#pragma unroll
      for (int part = 0; part < TC_N / 16; ++part) {
        float vv[16];
        tmem_ld16(tmem + trow + (uint32_t)(b * TC_N + part * 16), vv);
#pragma unroll
        for (int i = 0; i < 16; ++i) dst[(long long)(part * 16 + i) * lds] = vv[i];
        if (maxabs)
#pragma unroll
          for (int i = 0; i < 16; ++i) vmax = fmaxf(vmax, fabsf(vv[i]));
        if (ACC && dst2) {
          float a[16];
#pragma unroll
          for (int i = 0; i < 16; ++i) a[i] = dst2[(long long)(part * 16 + i) * lds];
          if (ACC == 2) {
            // (X0, X1) += D as a renormalised pair: X0 + (X1 + D) by an
            // error-free two-sum, so X1 stays below 2^-24 |X0| and the pair
            // keeps 48 bits however many corrections it collects
            float* dst0 = dst2 - (long long)d.nb * NB * lds;
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              const float x0 = dst0[(long long)(part * 16 + i) * lds];
              const float y = a[i] + vv[i];
              const float s = x0 + y, bb = s - x0;
              dst0[(long long)(part * 16 + i) * lds] = s;
              dst2[(long long)(part * 16 + i) * lds] = (x0 - (s - bb)) + (y - bb);
            }
          } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) dst2[(long long)(part * 16 + i) * lds] = a[i] + vv[i];
          }
        }
      }
      if (maxabs) {  // largest |result| of the system (non-negative FP32 bits order like integers)
        for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
        if (lane == 0) atomicMax(maxabs + blockIdx.y, __float_as_int(vmax));
      }
      tc_fence_before();
      mbar_arrive(&bar_tfree[b]);
      return true;
    };
    float vn[TC_KC];
    bool have_next = true;
    {
      const SweepChunk c = sweep_chunk(dir, d.nb, d.w, row_of(0), 0);
      load_chunk(c.jb, c.half, vn);
    }
    int epi_done = -1;  // last block row written to global memory
    long long g = 0;
    bool ok = true;
    for (int sidx = 0; sidx < nsteps && ok; ++sidx) {
      const int k = row_of(sidx);
      const int nchunk = sweep_nchunk(dir, d.nb, d.w, k);
      for (int q = 0; q < nchunk; ++q, ++g) {
        if (abort_flag) { ok = false; break; }
        // the previous row's results go out once two chunks of this row are queued
        // (and always before a chunk that reads them)
        const SweepChunk c = sweep_chunk(dir, d.nb, d.w, k, q);
        if (sidx > 0 && epi_done < sidx - 1 && (q == 2 || c.dep)) {
          if (!epilogue(sidx - 1)) { ok = false; break; }
          epi_done = sidx - 1;
        }
        if (!have_next) load_chunk(c.jb, c.half, vn);
        float v[TC_KC];
#pragma unroll
        for (int t = 0; t < TC_KC; ++t) v[t] = vn[t];
        // prefetch the next chunk unless it reads rows not yet written
        {
          int nk = k, nq = q + 1, ns = sidx;
          if (nq == nchunk) { ns = sidx + 1; nk = ns < nsteps ? row_of(ns) : -1; nq = 0; }
          have_next = false;
          if (nk >= 0) {
            const SweepChunk cn = sweep_chunk(dir, d.nb, d.w, nk, nq);
            if (!cn.dep || epi_done >= ns - 1) {
              load_chunk(cn.jb, cn.half, vn);
              have_next = true;
            }
          }
        }
        const int st = (int)(g % TC_STAGES);
        if (g >= TC_STAGES &&
            !mbar_wait(&bar_mma[st], (uint32_t)(((g - TC_STAGES) / TC_STAGES) & 1), limit)) { abort_flag = 1; ok = false; break; }
        float* ahi = sA + (st * 2 + 0) * TC_ACHUNK;
        float* alo = sA + (st * 2 + 1) * TC_ACHUNK;
        if (passes == 1) {
#pragma unroll
          for (int t4 = 0; t4 < TC_KC / 4; ++t4)
            *reinterpret_cast<float4*>(ahi + canon_off(tid, 4 * t4)) =
                make_float4(tf32_rna(v[4 * t4]), tf32_rna(v[4 * t4 + 1]), tf32_rna(v[4 * t4 + 2]),
                            tf32_rna(v[4 * t4 + 3]));
        } else {
#pragma unroll
          for (int t4 = 0; t4 < TC_KC / 4; ++t4) {
            float4 h, l;
            h.x = tf32_rna(v[4 * t4 + 0]); l.x = v[4 * t4 + 0] - h.x;
            h.y = tf32_rna(v[4 * t4 + 1]); l.y = v[4 * t4 + 1] - h.y;
            h.z = tf32_rna(v[4 * t4 + 2]); l.z = v[4 * t4 + 2] - h.z;
            h.w = tf32_rna(v[4 * t4 + 3]); l.w = v[4 * t4 + 3] - h.w;
            const int off = canon_off(tid, 4 * t4);
            *reinterpret_cast<float4*>(ahi + off) = h;
            *reinterpret_cast<float4*>(alo + off) = l;
          }
        }
        fence_async_smem();
        mbar_arrive(&bar_a[st]);
      }
      // a row with fewer than three chunks and no dependent chunk
      if (ok && sidx > 0 && epi_done < sidx - 1) {
        if (!epilogue(sidx - 1)) ok = false;
        else epi_done = sidx - 1;
      }
    }
    if (ok && epi_done < nsteps - 1) epilogue(nsteps - 1);
  }
  // wind-down: after an abort, wait (bounded) for work still in flight before freeing TMEM
  __syncthreads();
  if (tid == 0 && abort_flag) {
    const long long ql = last_commit;
    if (ql >= 0) mbar_wait(&bar_pfree[ql % TC_PST], (uint32_t)((ql / TC_PST) & 1));
    for (int s2 = 0; s2 < TC_PST; ++s2)
      if (tma_pending[s2] >= 0) mbar_wait(&bar_p[s2], (uint32_t)((tma_pending[s2] / TC_PST) & 1));
    atomicOr(err, DE_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TC_N));
}

constexpr size_t tc_smem_bytes() {
  return ((size_t)TC_STAGES * 2 * TC_ACHUNK + (size_t)TC_PST * TC_PCHUNK) * sizeof(float);
}

// ------------------------------------------------------------- panels
// Builds the forward and backward panels of a block-band factor (FP32):
// P_k[:, jj-th block] for block j = j0 + jj and Q_k[:, ii-th block] for block
// i = k + ii, each written as two 32-wide K chunks in canonical hi/lo form.
// grid (w+1, nb, batch), 256 threads; 64x64 SIMT products in FP32.
__global__ void __launch_bounds__(NT) k_make_panels(const BandDesc* __restrict__ bd, const TcDesc* __restrict__ td,
                                                    const float* __restrict__ lpool, float* __restrict__ ppool,
                                                    const BandDesc* __restrict__ bdb = nullptr) {
  const BandDesc d0 = bd[blockIdx.z];
  const BandDesc d1 = bdb ? bdb[blockIdx.z] : d0;  // backward panels: U^T of a general matrix, else L
  const TcDesc t = td[blockIdx.z];
  const int k = blockIdx.y, jj = blockIdx.x;
  if (k >= d0.nb) return;
  __shared__ __align__(16) float smA[SM_TILE];
  __shared__ __align__(16) float smB[SM_TILE];
  __shared__ float tile[NB][NB + 1];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int dir = 0; dir < 2; ++dir) {
    const BandDesc& d = dir == 0 ? d0 : d1;
    const float* Li = lpool + d.oLinv + (long long)k * NB * NB;
    int nblk = dir == 0 ? (k - (k - min(k, d.w)) + 1) : (min(d.w, d.nb - 1 - k) + 1);
    if (jj >= nblk) continue;
    float acc[4][4];
    tile_zero(acc);
    if (dir == 0) {
      int j = k - min(k, d.w) + jj;
      if (j == k) {
        for (int e = tid; e < NB * NB; e += NT) tile[e / NB][e % NB] = Li[e];
      } else {
        tile_gemm<float, false, false>(acc, Li, NB, lpool + band_block(d, k, j), NB, NB, smA, smB);
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int p = 0; p < 4; ++p) tile[ty * 4 + q][tx * 4 + p] = -acc[q][p];
      }
    } else {
      int i = k + jj;
      if (i == k) {
        for (int e = tid; e < NB * NB; e += NT) tile[e % NB][e / NB] = Li[e];  // transpose
      } else {
        // -Linv_kk^T L_ik^T = -(L_ik Linv_kk)^T
        tile_gemm<float, false, false>(acc, lpool + band_block(d, i, k), NB, Li, NB, NB, smA, smB);
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int p = 0; p < 4; ++p) tile[tx * 4 + p][ty * 4 + q] = -acc[q][p];
      }
    }
    __syncthreads();
    float* dst0 = ppool + panel_chunk(dir == 0 ? t.oPf : t.oPb, d.w, k, 2 * jj);
    for (int e = tid; e < NB * NB; e += NT) {
      int r = e / NB, c = e % NB;  // r = output row (N), c = K index within this block
      float v = tile[r][c];
      float h = tf32_rna(v);
      float* dst = dst0 + (c / TC_KC) * TC_PCHUNK;
      int off = canon_off(r, c % TC_KC);
      dst[off] = h;
      dst[TC_N * TC_KC + off] = v - h;
    }
    __syncthreads();
  }
}

// ------------------------------------------------- block Cholesky updates
// Right-looking-free block Cholesky with the trailing products on the tensor
// cores.  Step k of the left-looking factor needs, for the diagonal block and
// every block below it in column k,
//     C_ik = A_ik - sum_{j < k} L_ij L_kj^T        (i = k .. k + w)
// which is a contraction over the K range of block columns j.  Each finished
// block L_ij is stored once more as TF32 hi / lo operand tiles (k_chol_tile:
// two 32-wide K chunks, each a 64-row canonical K-major hi part then lo part,
// 8192 floats per block, at the block's band position), so that the update
// streams ready operands with cp.async.bulk and runs 3xTF32 MMAs (a_lo b_hi,
// a_hi b_lo, a_hi b_hi) with FP32 accumulation in TMEM.  One CTA updates two
// blocks (i0, i0 + 1) of column k: their tiles of block column j land side by
// side in shared memory as the M = 128 operand, the tile of L_kj is the N = 64
// operand.  The diagonal factor, the panel L_ik = C_ik Linv_kk^T and the
// tiling of the new column stay with k_chol_rl_diag / k_chol_rl_panel /
// k_chol_tile.
constexpr int CU_TILE = 4 * 2048;       // floats of one block's operand tiles (2 chunks x hi, lo)
constexpr int CU_HALF = 2048;           // floats of one 64-row x 32 hi (or lo) part
constexpr int CU_STAGES = 2;
constexpr int CU_STAGE = 6 * CU_HALF;   // A hi (2 halves), A lo (2 halves), B hi, B lo
constexpr int CU_THREADS = 192;         // warps 0-3 epilogue, 4 copies, 5 MMAs
constexpr size_t CU_SMEM = (size_t)CU_STAGES * CU_STAGE * sizeof(float);

__host__ __device__ __forceinline__ long long cu_tile(const BandDesc& d, long long toff, int i, int j) {
  return toff + ((long long)i * (d.w + 1) + (j - i + d.w)) * CU_TILE;
}

// operand tiles of the blocks (i, k), i = k .. k + w, of every system; grid (w + 1, systems)
__global__ void __launch_bounds__(256) k_chol_tile(const BandDesc* __restrict__ bd, const float* __restrict__ pool,
                                                   const long long* __restrict__ toff, float* __restrict__ tiles,
                                                   int k) {
  const BandDesc d = bd[blockIdx.y];
  const int i = k + blockIdx.x;
  if (k >= d.nb || i >= d.nb || i - k > d.w) return;
  const float* L = pool + band_block(d, i, k);
  float* t = tiles + cu_tile(d, toff[blockIdx.y], i, k);
  for (int e = threadIdx.x; e < NB * NB; e += 256) {
    const int r = e / NB, c = e % NB;
    const float v = L[e], h = tf32_rna(v);
    float* dst = t + (c / TC_KC) * 2 * CU_HALF + canon_off(r, c % TC_KC);
    dst[0] = h;
    dst[CU_HALF] = v - h;
  }
}

// C_ik = A_ik - sum_{j<k} L_ij L_kj^T for the block pair i0 = k + 2 blockIdx.x,
// i0 + 1 of every system (blockIdx.y); in place in the band pool
__global__ void __launch_bounds__(CU_THREADS, 1)
    k_chol_upd_tc(const BandDesc* __restrict__ bd, float* __restrict__ pool, const float* __restrict__ tiles,
                  const long long* __restrict__ toff, const float* __restrict__ zero_tile, int k,
                  int* __restrict__ err) {
  const BandDesc d = bd[blockIdx.y];
  const int i0 = k + 2 * blockIdx.x;
  if (k >= d.nb || i0 >= d.nb || i0 - k > d.w) return;
  const bool two = i0 + 1 < d.nb && i0 + 1 - k <= d.w;
  const int jlo = max(0, i0 - d.w), nch = 2 * (k - jlo);
  if (nch <= 0) return;
  const long long tb = toff[blockIdx.y];
  const long long limit = g_tc_wait_limit;
  extern __shared__ __align__(128) unsigned char cu_raw[];
  float* sm = reinterpret_cast<float*>(cu_raw);
  __shared__ __align__(8) uint64_t bar_full[CU_STAGES], bar_free[CU_STAGES], bar_done;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  __shared__ long long issued, mma_groups;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < CU_STAGES; ++s) { mbar_init(&bar_full[s], 1); mbar_init(&bar_free[s], 1); }
    mbar_init(&bar_done, 1);
    abort_flag = 0;
    issued = mma_groups = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(TC_N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  if (warp == 4) {
    // ------------------------------------------------ copies (one thread)
    if (lane == 0) {
      constexpr uint32_t hb = CU_HALF * 4;
      for (int q = 0; q < nch && !abort_flag; ++q) {
        const int st = q % CU_STAGES, j = jlo + q / 2, c = q & 1;
        if (q >= CU_STAGES && !mbar_wait(&bar_free[st], (uint32_t)(((q - CU_STAGES) / CU_STAGES) & 1), limit)) {
          abort_flag = 1;
          break;
        }
        float* dst = sm + st * CU_STAGE;
        const float* a0 = tiles + cu_tile(d, tb, i0, j) + c * 2 * CU_HALF;
        const float* a1 = (two && i0 + 1 - j <= d.w) ? tiles + cu_tile(d, tb, i0 + 1, j) + c * 2 * CU_HALF
                                                     : zero_tile;
        const float* b = tiles + cu_tile(d, tb, k, j) + c * 2 * CU_HALF;
        mbar_expect_tx(&bar_full[st], 6 * hb);
        bulk_g2s(dst + 0 * CU_HALF, a0, hb, &bar_full[st]);            // A hi, rows 0-63
        bulk_g2s(dst + 1 * CU_HALF, a1, hb, &bar_full[st]);            // A hi, rows 64-127
        bulk_g2s(dst + 2 * CU_HALF, a0 + CU_HALF, hb, &bar_full[st]);  // A lo
        bulk_g2s(dst + 3 * CU_HALF, a1 + CU_HALF, hb, &bar_full[st]);
        bulk_g2s(dst + 4 * CU_HALF, b, hb, &bar_full[st]);             // B hi
        bulk_g2s(dst + 5 * CU_HALF, b + CU_HALF, hb, &bar_full[st]);   // B lo
        issued = q + 1;
      }
    }
  } else if (warp == 5) {
    // ------------------------------------------------ MMAs (one thread)
    if (lane == 0) {
      constexpr uint32_t idesc = tc_idesc(TC_M, TC_N);
      for (int q = 0; q < nch && !abort_flag; ++q) {
        const int st = q % CU_STAGES;
        if (!mbar_wait(&bar_full[st], (uint32_t)((q / CU_STAGES) & 1), limit)) { abort_flag = 1; break; }
        tc_fence_after();
        const uint32_t a_hi = smem_u32(sm + st * CU_STAGE), a_lo = a_hi + 2 * CU_HALF * 4;
        const uint32_t b_hi = a_hi + 4 * CU_HALF * 4, b_lo = a_hi + 5 * CU_HALF * 4;
#pragma unroll
        for (int kk = 0; kk < TC_KC / 8; ++kk) {
          const uint32_t koff = kk * 2 * TC_LBO;
          mma_tf32(tmem, tc_desc(a_lo + koff), tc_desc(b_hi + koff), idesc, (q > 0 || kk > 0) ? 1u : 0u);
          mma_tf32(tmem, tc_desc(a_hi + koff), tc_desc(b_lo + koff), idesc, 1u);
          mma_tf32(tmem, tc_desc(a_hi + koff), tc_desc(b_hi + koff), idesc, 1u);
        }
        mma_commit(&bar_free[st]);
        mma_groups = q + 1;
      }
      mma_commit(&bar_done);
    }
  } else {
    // ------------------------------------------------ epilogue (128 threads)
    const int m = warp * 32 + lane;  // TMEM lane = row of the block pair
    const uint32_t trow = (uint32_t)(warp * 32) << 16;
    if (mbar_wait(&bar_done, 0u, limit) && !abort_flag) {
      tc_fence_after();
      const int blk = i0 + (m >> 6);
      float* A = (m < 64 || two) ? pool + band_block(d, blk, k) + (long long)(m & 63) * NB : nullptr;
#pragma unroll 1
      for (int part = 0; part < TC_N / 16; ++part) {
        float v[16];
        tmem_ld16(tmem + trow + (uint32_t)(part * 16), v);
        if (A) {
#pragma unroll
          for (int t4 = 0; t4 < 4; ++t4) {
            float4 a = *reinterpret_cast<float4*>(A + part * 16 + 4 * t4);
            a.x -= v[4 * t4]; a.y -= v[4 * t4 + 1]; a.z -= v[4 * t4 + 2]; a.w -= v[4 * t4 + 3];
            *reinterpret_cast<float4*>(A + part * 16 + 4 * t4) = a;
          }
        }
      }
    } else {
      abort_flag = 1;
    }
  }
  // wind-down: after an abort, wait (bounded) for copies and MMAs in flight before freeing TMEM
  __syncthreads();
  if (tid == 0 && abort_flag) {
    const long long qi = issued, qm = mma_groups;
    if (qm > 0) mbar_wait(&bar_free[(qm - 1) % CU_STAGES], (uint32_t)(((qm - 1) / CU_STAGES) & 1));
    for (long long q = qm; q < qi; ++q) mbar_wait(&bar_full[q % CU_STAGES], (uint32_t)((q / CU_STAGES) & 1));
    atomicOr(err, DE_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_N));
}

}  // namespace bddc
