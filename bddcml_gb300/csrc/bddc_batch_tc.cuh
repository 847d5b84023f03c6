// Batched working-precision products on the tensor cores (3xTF32, TMEM
// accumulation) for the FP32 preconditioner blocks of the batched solve:
//   out[o + r][c] = sum_j A[r][j] B[j][c],   r < m, c < nk
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
// Each A chunk is split into TF32 hi and lo on its way into tensor memory.  A
// B chunk is one canonical operand of 128 rows (b_hi in rows 0-63, b_lo in
// rows 64-127): per K step one MMA of N = 128, a_hi [b_hi | b_lo], and one of
// N = 64, a_lo b_hi, accumulate D_hi = a b_hi and D_lo = a_hi b_lo, and the
// epilogue adds the two halves in FP64 (Ootomo and Yokota's 3xTF32: the
// accuracy of an FP32 product).
//
// Persistent and warp-specialised, one CTA per SM over the job list:
//   warp 8  (one thread) moves A chunks into a ring of 9 slots (16 KB),
//   warp 10 (one thread) moves B chunks into a ring of 5 slots (16 KB),
//   warps 0-3 split the A chunks: thread r reads row r of the landed chunk
//           (which frees the slot at once), splits it and stores hi and lo
//           into tensor memory (4 buffers),
//   warp 9  (one thread) issues the MMAs, A from tensor memory and B from
//           shared memory, into one of two TMEM accumulators,
//   warps 4-7 read the finished accumulator and write the rows,
// so up to 144 KB of A stream from HBM per SM, the epilogue of one tile
// overlaps the main loop of the next, and shared memory carries only the
// landing copies, one read of A and the B operand reads.  A job may cover a K
// range of its tile (split K) and write its own partial rows.  Every wait is
// bounded; a timeout sets DE_TIMEOUT, and the CTA waits (bounded) for its
// copies and MMAs in flight before it frees TMEM and returns.
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

constexpr int GC_ASLOTS = 9;            // A landing slots
constexpr int GC_BSLOTS = 5;            // B landing slots
constexpr int GC_ABUF = 4;              // TMEM buffers of split A chunks
constexpr int GC_TILE = TC_M * TC_KC;   // floats of one A chunk, or of one B chunk (hi | lo)
constexpr int GC_BHALF = BMAX * TC_KC;  // floats of the hi (or lo) half of a B chunk
constexpr int GC_THREADS = 352;
constexpr int GC_PRODUCER_A = 8, GC_ISSUER = 9, GC_PRODUCER_B = 10;  // warps
// TMEM columns: two accumulators of 2 BMAX ([D_hi | D_lo]), then per A buffer
// TC_KC hi and TC_KC lo columns
constexpr int GC_N = 2 * BMAX;
constexpr uint32_t GC_ACOL = 2 * GC_N;
constexpr uint32_t GC_TCOLS = 512;
constexpr size_t GC_SMEM = (size_t)(GC_ASLOTS + GC_BSLOTS) * GC_TILE * sizeof(float) + 128;
static_assert(GC_BHALF * 2 == GC_TILE, "a B chunk is 64 columns x 32 K, hi and lo");
static_assert(GC_ACOL + GC_ABUF * 2 * TC_KC <= GC_TCOLS, "tensor memory columns");

// 32 consecutive TMEM columns of this warp's 32 lanes from 32 registers per thread
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float (&v)[32]) {
  uint32_t u[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) u[i] = __float_as_uint(v[i]);
  asm volatile("tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
               "{%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, %16, "
               "%17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32};"
               :
               : "r"(taddr),
               "r"(u[0]), "r"(u[1]), "r"(u[2]), "r"(u[3]),
               "r"(u[4]), "r"(u[5]), "r"(u[6]), "r"(u[7]),
               "r"(u[8]), "r"(u[9]), "r"(u[10]), "r"(u[11]),
               "r"(u[12]), "r"(u[13]), "r"(u[14]), "r"(u[15]),
               "r"(u[16]), "r"(u[17]), "r"(u[18]), "r"(u[19]),
               "r"(u[20]), "r"(u[21]), "r"(u[22]), "r"(u[23]),
               "r"(u[24]), "r"(u[25]), "r"(u[26]), "r"(u[27]),
               "r"(u[28]), "r"(u[29]), "r"(u[30]), "r"(u[31])
               : "memory");
}

__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// D (+)= A B with A (M x 8, TF32, one element per column) in tensor memory
__device__ __forceinline__ void mma_tf32_ta(uint32_t dtmem, uint32_t atmem, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(dtmem),
      "r"(atmem), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__global__ void __launch_bounds__(GC_THREADS, 1)
    kb_gemm_tc3(const TcJob* __restrict__ jobs, int njobs, const float* __restrict__ At,
                const float* __restrict__ Bt, double* out, int ldo, int nk,
                int* __restrict__ err, const int* __restrict__ ndone) {
  if (batch_all_done(ndone, nk)) return;
  extern __shared__ __align__(128) unsigned char gc_raw[];
  float* sA = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(gc_raw) + 127) & ~uintptr_t(127));
  float* sB = sA + GC_ASLOTS * GC_TILE;
  __shared__ __align__(8) uint64_t bar_afull[GC_ASLOTS], bar_afree[GC_ASLOTS];
  __shared__ __align__(8) uint64_t bar_bfull[GC_BSLOTS], bar_bempty[GC_BSLOTS];
  __shared__ __align__(8) uint64_t bar_a_full[GC_ABUF], bar_a_empty[GC_ABUF];
  __shared__ __align__(8) uint64_t bar_acc_full[2], bar_acc_empty[2];
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  __shared__ long long last_aload[GC_ASLOTS], last_bload[GC_BSLOTS], last_mma;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < GC_ASLOTS; ++s) {
      mbar_init(&bar_afull[s], 1);
      mbar_init(&bar_afree[s], TC_THREADS);
      last_aload[s] = -1;
    }
    for (int s = 0; s < GC_BSLOTS; ++s) {
      mbar_init(&bar_bfull[s], 1);
      mbar_init(&bar_bempty[s], 1);
      last_bload[s] = -1;
    }
    for (int s = 0; s < GC_ABUF; ++s) {
      mbar_init(&bar_a_full[s], TC_THREADS);
      mbar_init(&bar_a_empty[s], 1);
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
                 "r"(GC_TCOLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (warp == GC_PRODUCER_A || warp == GC_PRODUCER_B) {
    // ------------------------------------------------ bulk copies (one thread each for A and B)
    if (lane == 0) {
      const bool isA = warp == GC_PRODUCER_A;
      const int nslot = isA ? GC_ASLOTS : GC_BSLOTS;
      uint64_t* full = isA ? bar_afull : bar_bfull;
      uint64_t* release = isA ? bar_afree : bar_bempty;
      long long* last = isA ? last_aload : last_bload;
      float* ring = isA ? sA : sB;
      const float* src = isA ? At : Bt;
      long long q = 0;
      bool ok = true;
      for (int j = blockIdx.x; j < njobs && ok; j += gridDim.x) {
        const TcJob jb = jobs[j];
        const long long base = isA ? jb.a : jb.b;
        for (int c = 0; c < jb.nch; ++c, ++q) {
          const int s = (int)(q % nslot);
          const long long use = q / nslot;
          if (abort_flag || (use > 0 && !mbar_wait(&release[s], (uint32_t)((use - 1) & 1)))) {
            abort_flag = 1;
            ok = false;
            break;
          }
          mbar_expect_tx(&full[s], GC_TILE * (uint32_t)sizeof(float));
          bulk_g2s(ring + s * GC_TILE, src + base + (long long)c * GC_TILE, GC_TILE * sizeof(float), &full[s]);
          last[s] = q;
        }
      }
    }
  } else if (warp == GC_ISSUER) {
    // ------------------------------------------------ MMA issuer (one thread)
    if (lane == 0) {
      constexpr uint32_t idesc = tc_idesc(TC_M, GC_N);      // a_hi [b_hi | b_lo]
      constexpr uint32_t idesc_hi = tc_idesc(TC_M, BMAX);  // a_lo b_hi (rows 0-63 of the B chunk)
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
        const uint32_t dt = tmem + (uint32_t)(ab * GC_N);
        bool ok = true;
        for (int c = 0; c < nch; ++c, ++q) {
          const int sb = (int)(q % GC_BSLOTS), sa = (int)(q % GC_ABUF);
          if (abort_flag || !mbar_wait(&bar_a_full[sa], (uint32_t)((q / GC_ABUF) & 1)) ||
              !mbar_wait(&bar_bfull[sb], (uint32_t)((q / GC_BSLOTS) & 1))) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a_hi = tmem + GC_ACOL + (uint32_t)(sa * 2 * TC_KC), a_lo = a_hi + TC_KC;
          const uint32_t b = smem_u32(sB + sb * GC_TILE);
#pragma unroll
          for (int kk = 0; kk < TC_KC / 8; ++kk) {
            const uint32_t koff = kk * 2 * TC_LBO;
            const uint32_t acc = (c > 0 || kk > 0) ? 1u : 0u;
            mma_tf32_ta(dt, a_hi + kk * 8, tc_desc(b + koff), idesc, acc);
            mma_tf32_ta(dt, a_lo + kk * 8, tc_desc(b + koff), idesc_hi, 1u);
          }
          mma_commit(&bar_bempty[sb]);
          mma_commit(&bar_a_empty[sa]);
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
    // ------------------------------------------------ TF32 split of the A chunks into tensor memory
    // thread tid owns row tid of every chunk: eight 16-byte pieces of the
    // canonical order (a quarter-warp reads 128 contiguous bytes)
    long long q = 0;
    bool ok = true;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    for (int j = blockIdx.x; j < njobs && ok; j += gridDim.x) {
      const int nch = jobs[j].nch;
      for (int c = 0; c < nch; ++c, ++q) {
        const int s = (int)(q % GC_ASLOTS), sa = (int)(q % GC_ABUF);
        const long long ua = q / GC_ABUF;
        bool good = !abort_flag && mbar_wait(&bar_afull[s], (uint32_t)((q / GC_ASLOTS) & 1)) &&
                    (ua == 0 || mbar_wait(&bar_a_empty[sa], (uint32_t)((ua - 1) & 1)));
        good = __all_sync(0xffffffffu, good);  // the TMEM stores below are warp-collective
        if (!good) {
          abort_flag = 1;
          ok = false;
          break;
        }
        tc_fence_after();
        const float* a = sA + s * GC_TILE;
        float4 x[TC_KC / 4];
#pragma unroll
        for (int kq = 0; kq < TC_KC / 4; ++kq) x[kq] = *reinterpret_cast<const float4*>(a + canon_off(tid, 4 * kq));
        mbar_arrive(&bar_afree[s]);  // the row is in registers: the slot may take the next chunk
        float h[TC_KC], l[TC_KC];
#pragma unroll
        for (int kq = 0; kq < TC_KC / 4; ++kq) {
          h[4 * kq + 0] = tf32_rna(x[kq].x); l[4 * kq + 0] = tf32_rna(x[kq].x - h[4 * kq + 0]);
          h[4 * kq + 1] = tf32_rna(x[kq].y); l[4 * kq + 1] = tf32_rna(x[kq].y - h[4 * kq + 1]);
          h[4 * kq + 2] = tf32_rna(x[kq].z); l[4 * kq + 2] = tf32_rna(x[kq].z - h[4 * kq + 2]);
          h[4 * kq + 3] = tf32_rna(x[kq].w); l[4 * kq + 3] = tf32_rna(x[kq].w - h[4 * kq + 3]);
        }
        const uint32_t ta = tmem + lane_base + GC_ACOL + (uint32_t)(sa * 2 * TC_KC);
        tmem_st32(ta, h);
        tmem_st32(ta + TC_KC, l);
        tmem_st_wait();
        tc_fence_before();
        mbar_arrive(&bar_a_full[sa]);
      }
    }
  } else {
    // ------------------------------------------------ epilogue (warps 4-7 read TMEM lanes 32 (warp - 4) ..)
    const int ew = warp - 4;
    int t = 0;
    for (int j = blockIdx.x; j < njobs; j += gridDim.x, ++t) {
      const TcJob jb = jobs[j];
      const int ab = t & 1;
      bool good = !abort_flag && mbar_wait(&bar_acc_full[ab], (uint32_t)((t / 2) & 1));
      good = __all_sync(0xffffffffu, good);  // the TMEM loads below are warp-collective
      if (!good) {
        abort_flag = 1;
        break;
      }
      tc_fence_after();
      const uint32_t ta = tmem + ((uint32_t)(ew * 32) << 16) + (uint32_t)(ab * GC_N);
      const int r = ew * 32 + lane;
      double* orow = out + (jb.o + r) * ldo;
#pragma unroll 1
      for (int part = 0; part < BMAX / 16; ++part) {
        float wh[16], wl[16];
        tmem_ld16(ta + (uint32_t)(part * 16), wh);
        tmem_ld16(ta + (uint32_t)(BMAX + part * 16), wl);
        if (r < jb.m)
#pragma unroll
          for (int i = 0; i < 16; i += 2) {
            const int c = part * 16 + i;
            if (c < nk) {
              double2 y = make_double2((double)wh[i] + (double)wl[i], (double)wh[i + 1] + (double)wl[i + 1]);
              if (jb.nch == 0) y = make_double2(0.0, 0.0);
              *reinterpret_cast<double2*>(orow + c) = y;
            }
          }
      }
      tc_fence_before();
      mbar_arrive(&bar_acc_empty[ab]);  // the accumulator may take tile t + 2
    }
  }
  // wind-down: after an abort, wait (bounded) for the copies and MMAs in flight before freeing TMEM
  __syncthreads();
  if (tid == 0 && abort_flag) {
    for (int s = 0; s < GC_ASLOTS; ++s)
      if (last_aload[s] >= 0) mbar_wait(&bar_afull[s], (uint32_t)((last_aload[s] / GC_ASLOTS) & 1));
    for (int s = 0; s < GC_BSLOTS; ++s)
      if (last_bload[s] >= 0) mbar_wait(&bar_bfull[s], (uint32_t)((last_bload[s] / GC_BSLOTS) & 1));
    const long long qm = last_mma;
    if (qm >= 0) mbar_wait(&bar_bempty[qm % GC_BSLOTS], (uint32_t)((qm / GC_BSLOTS) & 1));
    atomicOr(err, DE_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(GC_TCOLS));
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
// Columns c >= nk and rows beyond the segment are zero.  256 threads per block.
__global__ void __launch_bounds__(256) kb_tile_b(int seg, const DevSub* __restrict__ ds, const long long* __restrict__ boff, int lg,
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
  constexpr int PER = GC_BHALF / 256;  // elements per thread (blockDim.x == 256)
  double v[PER];
#pragma unroll
  for (int i = 0; i < PER; ++i) {  // all loads in flight before the stores
    // a warp takes 8 columns x 4 K rows: 64-byte row pieces of x, and 32
    // distinct banks for the canonical stores
    const int e = threadIdx.x + 256 * i;
    const int c = ((e >> 5) & 7) * 8 + (e & 7), kk = (e >> 8) * 4 + ((e >> 3) & 3);
    const int j = ch * TC_KC + kk;
    v[i] = 0.0;
    if (j < K && c < nk) {
      const int g = base + j;
      v[i] = x[((long long)idx[g] << lg) + c];
      if (w) v[i] *= w[g];
    }
  }
#pragma unroll
  for (int i = 0; i < PER; ++i) {
    const int e = threadIdx.x + 256 * i;
    const int c = ((e >> 5) & 7) * 8 + (e & 7), kk = (e >> 8) * 4 + ((e >> 3) & 3);
    const float h = tf32_rna((float)v[i]);
    const int o = canon_off(c, kk);
    sh[o] = h;
    sh[GC_BHALF + o] = tf32_rna((float)(v[i] - (double)h));
  }
  __syncthreads();
  float4* dst = reinterpret_cast<float4*>(Bt + boff[blockIdx.y] + (long long)((seg == 1 ? 0 : n1) + ch) * GC_TILE);
  for (int p = threadIdx.x; p < GC_TILE / 4; p += 256) dst[p] = reinterpret_cast<const float4*>(sh)[p];
}

}  // namespace bddc
