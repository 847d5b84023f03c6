// Batched working-precision product on the tensor cores (3xTF32, TMEM
// accumulation) for the FP32 preconditioner blocks of the batched solve:
//   out[oo + r][c] = addend + sum_j A1[r][j] B1[ob + j][c] + sum_j A2[r][j] B2[ob2 + j][c],  c < nk
// with the operands of kb_gemm_t<float> (GemmDesc).  One CTA per 128-row tile
// of one product: MMA M = 128 (rows of A), N = 64 (columns), K = 8 per
// instruction; each FP32 operand is split into TF32 hi + lo while staging and
// D += a_lo b_hi + a_hi b_lo + a_hi b_hi (Ootomo and Yokota's 3xTF32, about
// the accuracy of the FP32 SIMT product it replaces).  Warps 0-3 stage K
// chunks of 32 into the canonical K-major layout (A rows read as 16-byte
// pieces, eight threads per 128-byte row segment; the column block of B is
// transposed on the way) and write the result; one thread of warp 4 issues the
// MMAs.  Every wait is bounded and reports DE_TIMEOUT.
#pragma once

#include "bddc_batch_kernels.cuh"
#include "bddc_tc.cuh"

namespace bddc {

constexpr int GC_STAGES = 2;         // canonical hi / lo operand stages read by the MMAs
constexpr int GC_RAW = 4;            // raw FP32 chunks in flight (cp.async ring)
constexpr int GC_AH = TC_M * TC_KC;   // floats of one A half (hi or lo) per stage
constexpr int GC_BH = BMAX * TC_KC;   // floats of one B half
constexpr int GC_THREADS = TC_THREADS + 32;
constexpr int GC_RLA = TC_KC + 4;     // padded row of the raw A chunk (conflict-free column reads)
constexpr int GC_RLB = BMAX + 8;      // padded K row of the raw B chunk
constexpr int GC_RA = TC_M * GC_RLA, GC_RB = TC_KC * GC_RLB;
constexpr size_t GC_SMEM =
    ((size_t)GC_STAGES * (2 * GC_AH + 2 * GC_BH) + (size_t)GC_RAW * (GC_RA + GC_RB)) * sizeof(float) + 1024;

__global__ void __launch_bounds__(GC_THREADS, 1)
    kb_gemm_tc3(const GemmDesc* __restrict__ gd, const float* __restrict__ A, const float* __restrict__ B1,
                const float* __restrict__ B2, int ldb, double* out, const double* addend, int ldo, int nk,
                int* __restrict__ err, const int* __restrict__ ndone) {
  if (batch_all_done(ndone, nk)) return;
  const GemmDesc d = gd[blockIdx.y];
  const int r0 = blockIdx.x * TC_M;
  if (r0 >= d.m) return;
  extern __shared__ __align__(1024) unsigned char gc_raw[];
  float* smem = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(gc_raw) + 1023) & ~uintptr_t(1023));
  float* sA = smem;                          // [stage][hi | lo][GC_AH]
  float* sB = smem + GC_STAGES * 2 * GC_AH;  // [stage][hi | lo][GC_BH]
  float* rA = sB + GC_STAGES * 2 * GC_BH;    // [raw stage][128 rows][GC_RLA] row-major
  float* rB = rA + GC_RAW * GC_RA;           // [raw stage][32 K rows][GC_RLB] row-major
  __shared__ __align__(8) uint64_t bar_a[GC_STAGES], bar_mma[GC_STAGES], bar_done;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  __shared__ long long last_commit;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n1 = (d.k1 + TC_KC - 1) / TC_KC, nch = n1 + (d.k2 + TC_KC - 1) / TC_KC;
  if (tid == 0) {
    for (int s = 0; s < GC_STAGES; ++s) { mbar_init(&bar_a[s], TC_THREADS); mbar_init(&bar_mma[s], 1); }
    mbar_init(&bar_done, 1);
    abort_flag = 0;
    last_commit = -1;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(BMAX));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (warp == TC_THREADS / 32) {
    // ------------------------------------------------ MMA issuer (one thread)
    if (lane == 0) {
      constexpr uint32_t idesc = tc_idesc(TC_M, BMAX);
      for (int g = 0; g < nch; ++g) {
        const int st = g % GC_STAGES;
        if (!mbar_wait(&bar_a[st], (uint32_t)((g / GC_STAGES) & 1))) { abort_flag = 1; break; }
        tc_fence_after();
        const uint32_t a_hi = smem_u32(sA + (st * 2 + 0) * GC_AH), a_lo = smem_u32(sA + (st * 2 + 1) * GC_AH);
        const uint32_t b_hi = smem_u32(sB + (st * 2 + 0) * GC_BH), b_lo = smem_u32(sB + (st * 2 + 1) * GC_BH);
#pragma unroll
        for (int kk = 0; kk < TC_KC / 8; ++kk) {
          const uint32_t koff = kk * 2 * TC_LBO;
          const uint32_t acc = (g > 0 || kk > 0) ? 1u : 0u;
          mma_tf32(tmem, tc_desc(a_lo + koff), tc_desc(b_hi + koff), idesc, acc);
          mma_tf32(tmem, tc_desc(a_hi + koff), tc_desc(b_lo + koff), idesc, 1u);
          mma_tf32(tmem, tc_desc(a_hi + koff), tc_desc(b_hi + koff), idesc, 1u);
        }
        mma_commit(&bar_mma[st]);
        last_commit = g;
      }
      mma_commit(&bar_done);
    }
  } else {
    // ------------------------------------------------ staging + epilogue (128 threads)
    // raw chunks move by cp.async (zero-filled outside the operands), GC_RAW - 1
    // of them ahead of the one being split into the canonical hi / lo stages
    auto load = [&](int g) {
      const int rs = g % GC_RAW;
      const bool seg1 = g < n1;
      const int kb = seg1 ? g * TC_KC : (g - n1) * TC_KC;
      const int K = seg1 ? d.k1 : d.k2;
      const float* Ab = A + (seg1 ? d.oA : d.oA2);
      const int lda = seg1 ? d.lda : d.lda2;
      const float* Bb = seg1 ? B1 + d.ob * ldb : B2 + d.ob2 * ldb;
#pragma unroll
      for (int i = 0; i < 8; ++i) {  // A: row e >> 3, 16-byte piece e & 7
        const int e = tid + TC_THREADS * i;
        const int r = e >> 3, k = kb + (e & 7) * 4;
        const int nb = (r0 + r < d.m && k < K) ? 4 * min(4, K - k) : 0;
        const float* src = nb ? Ab + (long long)(r0 + r) * lda + k : Ab;
        cp_async16(rA + rs * GC_RA + r * GC_RLA + (e & 7) * 4, src, nb);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {  // B: K row e >> 4, columns 4 (e & 15) .. +3
        const int e = tid + TC_THREADS * i;
        const int k = e >> 4, c = (e & 15) * 4;
        const int nb = (kb + k < K && c < nk) ? 16 : 0;
        const float* src = nb ? Bb + (long long)(kb + k) * ldb + c : Bb;
        cp_async16(rB + rs * GC_RB + k * GC_RLB + c, src, nb);
      }
    };
    auto split = [](float x, float& h, float& l) { h = tf32_rna(x); l = x - h; };
    bool ok = true;
#pragma unroll
    for (int q = 0; q < GC_RAW - 1; ++q) {
      if (q < nch) load(q);
      cp_async_commit();
    }
    for (int g = 0; g < nch && ok; ++g) {
      const int st = g % GC_STAGES, rs = g % GC_RAW;
      cp_async_wait<GC_RAW - 2>();  // chunk g has landed (this thread's part)
      // ... and everyone's; everyone has also finished splitting chunk g - 1,
      // so its raw slot may take chunk g + GC_RAW - 1
      asm volatile("bar.sync 1, %0;" ::"r"(TC_THREADS) : "memory");
      if (g + GC_RAW - 1 < nch) load(g + GC_RAW - 1);
      cp_async_commit();
      if (g >= GC_STAGES &&
          !mbar_wait(&bar_mma[st], (uint32_t)(((g - GC_STAGES) / GC_STAGES) & 1))) { abort_flag = 1; ok = false; break; }
      float* ahi = sA + (st * 2 + 0) * GC_AH;
      float* alo = sA + (st * 2 + 1) * GC_AH;
      float* bhi = sB + (st * 2 + 0) * GC_BH;
      float* blo = sB + (st * 2 + 1) * GC_BH;
      const float* ra = rA + rs * GC_RA;
      const float* rb = rB + rs * GC_RB;
      // A: a quarter-warp takes 8 consecutive rows of one 16-byte column piece,
      // so both the padded raw reads and the canonical stores are conflict-free
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int e = tid + TC_THREADS * i;
        const int r = (e >> 6) * 8 + (e & 7), q = (e >> 3) & 7;
        const float4 x = *reinterpret_cast<const float4*>(ra + r * GC_RLA + q * 4);
        const int off = canon_off(r, q * 4);
        float4 h, l;
        split(x.x, h.x, l.x); split(x.y, h.y, l.y); split(x.z, h.z, l.z); split(x.w, h.w, l.w);
        *reinterpret_cast<float4*>(ahi + off) = h;
        *reinterpret_cast<float4*>(alo + off) = l;
      }
      // B (transposed): a warp takes 8 columns x 4 K rows, distinct banks for the
      // padded raw reads and for the canonical stores
      {
        const int nlo = lane & 7, klo = lane >> 3;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int blk = warp * 16 + i;  // 64 blocks of 8 columns x 4 K rows
          const int n = (blk & 7) * 8 + nlo, k = (blk >> 3) * 4 + klo;
          float h, l;
          split(rb[k * GC_RLB + n], h, l);
          bhi[canon_off(n, k)] = h;
          blo[canon_off(n, k)] = l;
        }
      }
      fence_async_smem();
      mbar_arrive(&bar_a[st]);
    }
    cp_async_wait<0>();
    // epilogue: row r0 + 32 warp + lane of the tile, 64 columns from TMEM
    if (ok && !abort_flag && mbar_wait(&bar_done, 0u)) {
      tc_fence_after();
      const int r = r0 + warp * 32 + lane;
      const uint32_t trow = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
      for (int part = 0; part < BMAX / 16; ++part) {
        float v[16];
        tmem_ld16(tmem + trow + (uint32_t)(part * 16), v);
        if (nch == 0)
#pragma unroll
          for (int i = 0; i < 16; ++i) v[i] = 0.f;
        if (r < d.m)
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int c = part * 16 + i;
            if (c < nk) {
              const long long o = (d.oo + r) * ldo + c;
              out[o] = addend ? addend[o] + (double)v[i] : (double)v[i];
            }
          }
      }
    } else {
      abort_flag = 1;
    }
  }
  // wind-down: after an abort, wait (bounded) for the MMAs in flight before freeing TMEM
  __syncthreads();
  if (tid == 0 && abort_flag) {
    const long long ql = last_commit;
    if (ql >= 0) mbar_wait(&bar_mma[ql % GC_STAGES], (uint32_t)((ql / GC_STAGES) & 1));
    atomicOr(err, DE_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BMAX));
}

}  // namespace bddc
