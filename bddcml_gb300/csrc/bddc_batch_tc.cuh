// Batched working-precision products on the tensor cores (3xTF32, TMEM
// accumulation) for the FP32 preconditioner blocks of the batched solve:
//   out[o + r][c] = addend + sum_j A[r][j] B[j][c],   r < m, c < nk
// for a list of jobs, each one 128-row tile of one subdomain product
// ([Z | Phi] with [W r ; u_c], or Phi^T with W r).
//
// Operands are laid out for the kernel once:
//  * A tiles (batch setup): every 128 x 32 chunk of A is one 16 KB block in
//    the canonical K-major no-swizzle order of the MMA (rows and K beyond the
//    matrix are zero), so one cp.async.bulk moves it;
//  * B chunks (every application, kb_tile_b): the 32 x 64 chunk of the
//    right-hand sides, split into TF32 hi and lo and transposed to the same
//    order, 16 KB per chunk.
// The A chunk is split into hi and lo in shared memory, in place, each thread
// on its own 16-byte pieces, and D += a_lo b_hi + a_hi b_lo + a_hi b_hi
// (Ootomo and Yokota's 3xTF32, the accuracy of an FP32 product).
//
// Persistent and warp-specialised, one CTA per SM over the job list:
//   warp 8  (one thread) issues the bulk copies into a 4-stage ring,
//   warps 0-3 split the A chunks,
//   warp 9  (one thread) issues the MMAs into one of two TMEM accumulators,
//   warps 4-7 read the finished accumulator and write the rows,
// so the epilogue of one tile overlaps the main loop of the next.  Every
// wait is bounded; a timeout sets DE_TIMEOUT, and the CTA waits (bounded) for
// its copies and MMAs in flight before it frees TMEM and returns.
#pragma once

#include "bddc_batch_kernels.cuh"
#include "bddc_tc.cuh"

namespace bddc {

// One 128-row output tile: A chunks at a, a + GC_TILE, ...; B chunks at b, ...
struct TcJob {
  long long a, b;  // float offsets of the first A chunk and of the first B chunk
  long long o;     // output row of tile row 0
  int m, nch;      // valid rows (<= TC_M), K chunks
};

constexpr int GC_STAGES = 4;
constexpr int GC_TILE = TC_M * TC_KC;   // floats of one A chunk, or of one B chunk (hi | lo)
constexpr int GC_BHALF = BMAX * TC_KC;  // floats of the hi (or lo) half of a B chunk
constexpr int GC_STAGE = 3 * GC_TILE;   // A (split in place into hi) | A lo | B hi, lo
constexpr int GC_THREADS = 320;
constexpr int GC_PRODUCER = 8, GC_ISSUER = 9;  // warps
constexpr size_t GC_SMEM = (size_t)GC_STAGES * GC_STAGE * sizeof(float) + 1024;
static_assert(GC_BHALF * 2 == GC_TILE, "a B chunk is 64 columns x 32 K, hi and lo");

__global__ void __launch_bounds__(GC_THREADS, 1)
    kb_gemm_tc3(const TcJob* __restrict__ jobs, int njobs, const float* __restrict__ At,
                const float* __restrict__ Bt, double* out, const double* addend, int ldo, int nk,
                int* __restrict__ err, const int* __restrict__ ndone) {
  if (batch_all_done(ndone, nk)) return;
  extern __shared__ __align__(1024) unsigned char gc_raw[];
  float* smem = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(gc_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t bar_full[GC_STAGES], bar_split[GC_STAGES], bar_empty[GC_STAGES];
  __shared__ __align__(8) uint64_t bar_acc_full[2], bar_acc_empty[2];
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  __shared__ long long last_load[GC_STAGES], last_mma;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < GC_STAGES; ++s) {
      mbar_init(&bar_full[s], 1);
      mbar_init(&bar_split[s], TC_THREADS);
      mbar_init(&bar_empty[s], 1);
      last_load[s] = -1;
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&bar_acc_full[b], 1);
      mbar_init(&bar_acc_empty[b], TC_THREADS);
    }
    abort_flag = 0;
    last_mma = -1;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(2 * BMAX));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (warp == GC_PRODUCER) {
    // ------------------------------------------------ bulk copies (one thread)
    if (lane == 0) {
      long long q = 0;
      bool ok = true;
      for (int j = blockIdx.x; j < njobs && ok; j += gridDim.x) {
        const TcJob jb = jobs[j];
        for (int c = 0; c < jb.nch; ++c, ++q) {
          const int s = (int)(q % GC_STAGES);
          const long long use = q / GC_STAGES;
          if (abort_flag || (use > 0 && !mbar_wait(&bar_empty[s], (uint32_t)((use - 1) & 1)))) {
            abort_flag = 1;
            ok = false;
            break;
          }
          float* st = smem + s * GC_STAGE;
          mbar_expect_tx(&bar_full[s], 2 * GC_TILE * (uint32_t)sizeof(float));
          bulk_g2s(st, At + jb.a + (long long)c * GC_TILE, GC_TILE * sizeof(float), &bar_full[s]);
          bulk_g2s(st + 2 * GC_TILE, Bt + jb.b + (long long)c * GC_TILE, GC_TILE * sizeof(float), &bar_full[s]);
          last_load[s] = q;
        }
      }
    }
  } else if (warp == GC_ISSUER) {
    // ------------------------------------------------ MMA issuer (one thread)
    if (lane == 0) {
      constexpr uint32_t idesc = tc_idesc(TC_M, BMAX);
      long long q = 0;
      int t = 0;
      for (int j = blockIdx.x; j < njobs; j += gridDim.x, ++t) {
        const int nch = jobs[j].nch;
        const int ab = t & 1;
        if (abort_flag || (t >= 2 && !mbar_wait(&bar_acc_empty[ab], (uint32_t)((t / 2 - 1) & 1)))) {
          abort_flag = 1;
          break;
        }
        tc_fence_after();
        const uint32_t dt = tmem + (uint32_t)(ab * BMAX);
        bool ok = true;
        for (int c = 0; c < nch; ++c, ++q) {
          const int s = (int)(q % GC_STAGES);
          if (abort_flag || !mbar_wait(&bar_split[s], (uint32_t)((q / GC_STAGES) & 1))) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a_hi = smem_u32(smem + s * GC_STAGE), a_lo = a_hi + GC_TILE * 4;
          const uint32_t b_hi = a_hi + 2 * GC_TILE * 4, b_lo = b_hi + GC_BHALF * 4;
#pragma unroll
          for (int kk = 0; kk < TC_KC / 8; ++kk) {
            const uint32_t koff = kk * 2 * TC_LBO;
            const uint32_t acc = (c > 0 || kk > 0) ? 1u : 0u;
            mma_tf32(dt, tc_desc(a_lo + koff), tc_desc(b_hi + koff), idesc, acc);
            mma_tf32(dt, tc_desc(a_hi + koff), tc_desc(b_lo + koff), idesc, 1u);
            mma_tf32(dt, tc_desc(a_hi + koff), tc_desc(b_hi + koff), idesc, 1u);
          }
          mma_commit(&bar_empty[s]);
          last_mma = q;
        }
        if (!ok) {
          abort_flag = 1;
          break;
        }
        mma_commit(&bar_acc_full[ab]);
      }
    }
  } else if (warp < 4) {
    // ------------------------------------------------ in-place TF32 split of the A chunks
    long long q = 0;
    bool ok = true;
    for (int j = blockIdx.x; j < njobs && ok; j += gridDim.x) {
      const int nch = jobs[j].nch;
      for (int c = 0; c < nch; ++c, ++q) {
        const int s = (int)(q % GC_STAGES);
        if (abort_flag || !mbar_wait(&bar_full[s], (uint32_t)((q / GC_STAGES) & 1))) {
          abort_flag = 1;
          ok = false;
          break;
        }
        float* ahi = smem + s * GC_STAGE;
        float* alo = ahi + GC_TILE;
#pragma unroll
        for (int i = 0; i < GC_TILE / 4 / TC_THREADS; ++i) {
          const int p = (tid + TC_THREADS * i) * 4;
          const float4 x = *reinterpret_cast<const float4*>(ahi + p);
          float4 h, l;
          h.x = tf32_rna(x.x); l.x = tf32_rna(x.x - h.x);
          h.y = tf32_rna(x.y); l.y = tf32_rna(x.y - h.y);
          h.z = tf32_rna(x.z); l.z = tf32_rna(x.z - h.z);
          h.w = tf32_rna(x.w); l.w = tf32_rna(x.w - h.w);
          *reinterpret_cast<float4*>(ahi + p) = h;
          *reinterpret_cast<float4*>(alo + p) = l;
        }
        fence_async_smem();
        mbar_arrive(&bar_split[s]);
      }
    }
  } else {
    // ------------------------------------------------ epilogue (warps 4-7 read TMEM lanes 32 (warp - 4) ..)
    const int ew = warp - 4;
    int t = 0;
    for (int j = blockIdx.x; j < njobs; j += gridDim.x, ++t) {
      const TcJob jb = jobs[j];
      const int ab = t & 1;
      if (abort_flag || !mbar_wait(&bar_acc_full[ab], (uint32_t)((t / 2) & 1))) {
        abort_flag = 1;
        break;
      }
      tc_fence_after();
      float v[BMAX];
      const uint32_t ta = tmem + ((uint32_t)(ew * 32) << 16) + (uint32_t)(ab * BMAX);
#pragma unroll
      for (int part = 0; part < BMAX / 16; ++part) {
        float w[16];
        tmem_ld16(ta + (uint32_t)(part * 16), w);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[part * 16 + i] = jb.nch > 0 ? w[i] : 0.f;
      }
      tc_fence_before();
      mbar_arrive(&bar_acc_empty[ab]);  // the accumulator may take tile t + 2
      const int r = ew * 32 + lane;
      if (r < jb.m) {
        double* orow = out + (jb.o + r) * ldo;
        const double* arow = addend ? addend + (jb.o + r) * ldo : nullptr;
#pragma unroll
        for (int c = 0; c < BMAX; c += 2)
          if (c < nk) {
            double2 y = make_double2((double)v[c], (double)v[c + 1]);
            if (arow) {
              y.x += arow[c];
              y.y += arow[c + 1];
            }
            *reinterpret_cast<double2*>(orow + c) = y;
          }
      }
    }
  }
  // wind-down: after an abort, wait (bounded) for the copies and MMAs in flight before freeing TMEM
  __syncthreads();
  if (tid == 0 && abort_flag) {
    for (int s = 0; s < GC_STAGES; ++s)
      if (last_load[s] >= 0) mbar_wait(&bar_full[s], (uint32_t)((last_load[s] / GC_STAGES) & 1));
    const long long qm = last_mma;
    if (qm >= 0) mbar_wait(&bar_empty[qm % GC_STAGES], (uint32_t)((qm / GC_STAGES) & 1));
    atomicOr(err, DE_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BMAX));
}

// A tiles of [A1 | A2] for every descriptor: tile (rt, ch) of descriptor y at
// toff[y] + (rt * nch + ch) * GC_TILE, nch = ceil(k1 / 32) + ceil(k2 / 32).
// One block per tile; each thread writes whole 16-byte pieces of the
// canonical order (piece p holds row (p >> 6) * 8 + (p & 7), K 4 ((p >> 3) & 7) ..).
__global__ void kb_tile_a(const GemmDesc* __restrict__ gd, const long long* __restrict__ toff,
                          const float* __restrict__ A, float* __restrict__ At) {
  const GemmDesc d = gd[blockIdx.y];
  const int n1 = (d.k1 + TC_KC - 1) / TC_KC, nch = n1 + (d.k2 + TC_KC - 1) / TC_KC;
  const int nrt = (d.m + TC_M - 1) / TC_M;
  const int ti = blockIdx.x;
  if (ti >= nrt * nch) return;
  const int rt = ti / nch, ch = ti % nch;
  const bool seg1 = ch < n1;
  const int K = seg1 ? d.k1 : d.k2, kb = (seg1 ? ch : ch - n1) * TC_KC, lda = seg1 ? d.lda : d.lda2;
  const float* Ab = A + (seg1 ? d.oA : d.oA2);
  float4* dst = reinterpret_cast<float4*>(At + toff[blockIdx.y] + (long long)ti * GC_TILE);
  for (int p = threadIdx.x; p < GC_TILE / 4; p += blockDim.x) {
    const int r = rt * TC_M + (p >> 6) * 8 + (p & 7), k = kb + ((p >> 3) & 7) * 4;
    float v[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) v[e] = (r < d.m && k + e < K) ? Ab[(long long)r * lda + k + e] : 0.f;
    dst[p] = make_float4(v[0], v[1], v[2], v[3]);
  }
}

// B chunks of one application: chunk ch of subdomain y at boff[y] + ch * GC_TILE,
// TF32 hi then lo, each 64 columns x 32 K in the canonical order.
//   seg 1 (chunks 0 .. ceil(ni / 32) - 1):   B[j][c] = w[rep + j] x[idx[rep + j]][c]
//   seg 2 (the next ceil(nc / 32) chunks):   B[j][c] = x[idx[coff + j]][c]
// Columns c >= nk and rows beyond the segment are zero.
__global__ void kb_tile_b(int seg, const DevSub* __restrict__ ds, const long long* __restrict__ boff, int lg,
                          const int* __restrict__ idx, const double* __restrict__ w, const double* __restrict__ x,
                          float* __restrict__ Bt, const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const DevSub s = ds[blockIdx.y];
  const int n1 = (s.ni + TC_KC - 1) / TC_KC;
  const int K = seg == 1 ? s.ni : s.nc, base = seg == 1 ? s.rep : s.coff;
  const int ch = blockIdx.x;
  if (ch * TC_KC >= K) return;
  __shared__ __align__(16) float sh[GC_TILE];
  for (int e = threadIdx.x; e < GC_BHALF; e += blockDim.x) {
    const int kk = e >> 6, c = e & 63;  // 64 consecutive threads read one row of x
    const int j = ch * TC_KC + kk;
    double v = 0.0;
    if (j < K && c < nk) {
      const int g = base + j;
      v = x[((long long)idx[g] << lg) + c];
      if (w) v *= w[g];
    }
    const float h = tf32_rna((float)v);
    const int o = canon_off(c, kk);
    sh[o] = h;
    sh[GC_BHALF + o] = tf32_rna((float)(v - (double)h));
  }
  __syncthreads();
  float4* dst = reinterpret_cast<float4*>(Bt + boff[blockIdx.y] + (long long)((seg == 1 ? 0 : n1) + ch) * GC_TILE);
  for (int p = threadIdx.x; p < GC_TILE / 4; p += blockDim.x) dst[p] = reinterpret_cast<const float4*>(sh)[p];
}

}  // namespace bddc
