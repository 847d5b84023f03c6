// Batched Schur apply Y = S X (and, with the FP32 preconditioner blocks as A,
// the preconditioner products of the batched solve; see the end of the file)
// with FP64-class accuracy on the bf16 tensor
// cores (tcgen05 kind::f16), by error-free slicing of both operands (Ozaki,
// Ogita, Oishi and Rump, "Error-free transformations of matrix
// multiplication by using fast routines of matrix multiplication and its
// applications", Numer. Algorithms 59, 2012).
//
// Every row i of S is scaled by 2^-e_i (|S_ij| < 2^e_i) and every column k of
// X by 2^-f_k, then cut into OZ_NS signed integer slices of 6 bits:
//     S_ij = 2^e_i sum_s sigma_s[i][j] 2^(-6 s),   X_jk = 2^f_k sum_t tau_t[j][k] 2^(-6 t),
// |sigma_1|, |tau_1| <= 64 and all later slices <= 32, all exact in bf16.
// Products of slices are integers, so for each diagonal d = s + t the sum
//     D_d[i][k] = sum_{s+t=d} sum_j sigma_s[i][j] tau_t[j][k]
// is an integer; with K <= OZ_KMAX the first three diagonals (d = 2, 3, 4)
// stay below 2^24 and are exact in the FP32 accumulators; the later ones are
// scaled by 2^-30 and less, so their FP32 rounding is below 2^-42 of the
// result.  Then Y_ik = 2^(e_i + f_k) sum_{d=2..9} D_d 2^(-6 d), summed in
// double-float.  Pairs with s + t > 9 are dropped (below 2^-54 per term).
//
// Tensor-core mapping: one CTA per (128-row tile, subdomain); D_d for
// d = 2..9 are eight 128 x 64 FP32 accumulators side by side in TMEM (all 512
// columns).  The eight X slices of a K chunk are stacked along N (N row
// 64 (t-1) + k), so one MMA with A = sigma_s and B = [tau_1 .. tau_4] writes
// D_{s+1} .. D_{s+4} at once (N = 256), and every K step of 16 needs 12 MMAs
// for the 36 slice pairs.  S slices are precomputed in the canonical K-major
// layout (core matrices of 8 rows x 16 bytes), X slices are made per apply;
// both are moved by cp.async.bulk, one elected thread issues the copies,
// another the MMAs, four warps read the accumulators at the end.
#pragma once

#include <cuda_bf16.h>

#include "bddc_batch_kernels.cuh"
#include "bddc_tc.cuh"

namespace bddc {

constexpr int OZ_NS = 8;                      // slices per operand
constexpr int OZ_M = 128;                     // rows per tile (MMA M)
constexpr int OZ_KC = 64;                     // K per chunk (bf16): 128-byte row pieces
constexpr int OZ_AB = OZ_M * OZ_KC;           // bf16 elements of one S slice block (16 KB)
constexpr int OZ_BB = OZ_NS * BMAX * OZ_KC;   // bf16 elements of one X chunk block, all slices (64 KB)
constexpr int OZ_ASTAGES = 4;
constexpr int OZ_KMAX = 3264;                 // exact leading diagonals up to this K (5120 * K < 2^24)
constexpr int OZ_THREADS = 192;               // warps 0-3 epilogue, 4 copies, 5 MMAs
constexpr size_t OZ_SMEM = (size_t)(2 * OZ_BB + OZ_ASTAGES * OZ_AB) * 2 + 1024;

// element offset of (row r, k) in a canonical K-major block of OZ_KC columns:
// core matrices of 8 rows x 8 bf16, 64 elements (128 B) apart along K,
// 8-row groups 512 elements (1024 B) apart
__host__ __device__ __forceinline__ int oz_off(int r, int k) { return (r >> 3) * 512 + (k >> 3) * 64 + (r & 7) * 8 + (k & 7); }

// instruction descriptor: kind::f16 with A = B = bf16, D = F32, both K-major
__host__ __device__ constexpr uint32_t oz_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// N slices of v = hi + lo, |v| <= 1: v ~ sum_s q_s 2^(-6 s), q_s integers
template <int N>
__device__ __forceinline__ void oz_split(float hi, float lo, float (&q)[N]) {
#pragma unroll
  for (int s = 0; s < N; ++s) {
    hi *= 64.f;
    lo *= 64.f;
    const float r = rintf(hi);
    q[s] = r;
    two_sum(hi - r, lo, hi, lo);
  }
}

// exponent e with |v| < 2^e for the largest magnitude v of a row or column
__device__ __forceinline__ int oz_exp(double vmax) {
  int e = 0;
  if (vmax > 0.0) frexp(vmax, &e);
  return e;
}

// ------------------------------------------------------- S slices (setup)
// erow[ro + r] for the rows of each subdomain's tiles: warp per row
__global__ void kb_oz_row_exp(const DevSub* __restrict__ ds, const float2* __restrict__ Spool,
                              const long long* __restrict__ eoff, int* __restrict__ erow) {
  const DevSub d = ds[blockIdx.y];
  const int r = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  const int nrow = (d.ni + OZ_M - 1) / OZ_M * OZ_M;
  if (r >= nrow) return;
  float m = 0.f;
  if (r < d.ni)
    for (int j = lane; j < d.ni; j += 32) m = fmaxf(m, fabsf(Spool[d.oS + (long long)r * d.NI + j].x));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  // |hi + lo| <= |hi| (1 + 2^-24): one more binade keeps every scaled entry within 1
  if (lane == 0) erow[eoff[blockIdx.y] + r] = oz_exp((double)m) + (m > 0.f ? 1 : 0);
}

// S slice blocks: block (tile rt, chunk c, slice s) at soff + ((rt * nch + c) * OZ_NS + s) * OZ_AB;
// grid (nch * nrt, nsub), 256 threads, 8 consecutive k per thread task
__global__ void __launch_bounds__(256) kb_oz_slice_s(const DevSub* __restrict__ ds, const float2* __restrict__ Spool,
                                                     const long long* __restrict__ soff,
                                                     const long long* __restrict__ eoff, const int* __restrict__ erow,
                                                     __nv_bfloat16* __restrict__ sl) {
  const DevSub d = ds[blockIdx.y];
  const int nch = (d.ni + OZ_KC - 1) / OZ_KC, nrt = (d.ni + OZ_M - 1) / OZ_M;
  if ((int)blockIdx.x >= nch * nrt) return;
  const int rt = blockIdx.x / nch, c = blockIdx.x % nch;
  __nv_bfloat16* base = sl + soff[blockIdx.y] + ((long long)rt * nch + c) * OZ_NS * OZ_AB;
  for (int task = threadIdx.x; task < OZ_M * (OZ_KC / 8); task += 256) {
    const int r = task / (OZ_KC / 8), k0 = (task % (OZ_KC / 8)) * 8;
    const int gr = rt * OZ_M + r;
    const float sc = ldexpf(1.f, -erow[eoff[blockIdx.y] + gr]);
    __align__(16) __nv_bfloat16 out[OZ_NS][8];
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
      const int gk = c * OZ_KC + k0 + kk;
      float2 a = make_float2(0.f, 0.f);
      if (gr < d.ni && gk < d.ni) a = Spool[d.oS + (long long)gr * d.NI + gk];
      float q[OZ_NS];
      oz_split(a.x * sc, a.y * sc, q);
#pragma unroll
      for (int s = 0; s < OZ_NS; ++s) out[s][kk] = __float2bfloat16_rn(q[s]);
    }
#pragma unroll
    for (int s = 0; s < OZ_NS; ++s)
      *reinterpret_cast<uint4*>(base + (long long)s * OZ_AB + oz_off(r, k0)) = *reinterpret_cast<const uint4*>(out[s]);
  }
}

// ------------------------------------------------------ X slices (per apply)
// The sliced vectors of a subdomain: mode 0 its interface (entries rep .. rep + ni,
// the product's K range for S, Z and Phi^T), mode 1 its constraints (coff ..
// coff + nc, the K range for Phi).  Entry j of column k is
// w[base + j] * x[idx[base + j] * nk + k] (w omitted: 1).
__device__ __forceinline__ void oz_range(const DevSub& d, int mode, int& base, int& cnt) {
  base = mode ? d.coff : d.rep;
  cnt = mode ? d.nc : d.ni;
}

// fcol[sub * BMAX + k] = exponent of the largest |entry| of column k
__global__ void __launch_bounds__(256) kb_oz_col_exp(const DevSub* __restrict__ ds, int lg, int mode,
                                                     const int* __restrict__ idx, const double* __restrict__ w,
                                                     const double* __restrict__ x, int* __restrict__ fcol,
                                                     const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const DevSub d = ds[blockIdx.x];
  int base, cnt;
  oz_range(d, mode, base, cnt);
  __shared__ double sh[256];
  const int k = threadIdx.x & (nk - 1), rl = threadIdx.x >> lg, nrl = 256 >> lg;
  double m = 0.0;
  for (int j = rl; j < cnt; j += nrl) {
    const double v = x[((long long)idx[base + j] << lg) + k];
    m = fmax(m, fabs(w ? w[base + j] * v : v));
  }
  sh[threadIdx.x] = m;
  __syncthreads();
  for (int st = 128; st >= nk; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + st]);
    __syncthreads();
  }
  if (threadIdx.x < nk) fcol[blockIdx.x * BMAX + threadIdx.x] = oz_exp(sh[threadIdx.x]);
}

// X chunk blocks of every subdomain: block c at xoff + c * OZ_BB, N row 64 s + k;
// grid (max chunks, nsub), 256 threads
__global__ void __launch_bounds__(256) kb_oz_slice_x(const DevSub* __restrict__ ds, int lg, int mode,
                                                     const int* __restrict__ idx, const double* __restrict__ w,
                                                     const double* __restrict__ x, const int* __restrict__ fcol,
                                                     const long long* __restrict__ xoff,
                                                     __nv_bfloat16* __restrict__ xl, const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const DevSub d = ds[blockIdx.y];
  int base, cnt;
  oz_range(d, mode, base, cnt);
  const int c = blockIdx.x;
  if (c * OZ_KC >= cnt) return;
  __shared__ double tile[OZ_KC][BMAX + 1];
  for (int e = threadIdx.x; e < OZ_KC * BMAX; e += 256) {
    const int j = e / BMAX, k = e % BMAX, gj = c * OZ_KC + j;
    double v = 0.0;
    if (k < nk && gj < cnt) {
      v = x[((long long)idx[base + gj] << lg) + k];
      if (w) v *= w[base + gj];
    }
    tile[j][k] = v;
  }
  __syncthreads();
  __nv_bfloat16* out0 = xl + xoff[blockIdx.y] + (long long)c * OZ_BB;
  for (int task = threadIdx.x; task < BMAX * (OZ_KC / 8); task += 256) {
    const int k = task / (OZ_KC / 8), j0 = (task % (OZ_KC / 8)) * 8;
    const double sc = ldexp(1.0, -fcol[blockIdx.y * BMAX + k]);
    __align__(16) __nv_bfloat16 out[OZ_NS][8];
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) {
      const double v = tile[j0 + jj][k] * sc;
      const float h = (float)v;
      float q[OZ_NS];
      oz_split(h, (float)(v - (double)h), q);
#pragma unroll
      for (int s = 0; s < OZ_NS; ++s) out[s][jj] = __float2bfloat16_rn(q[s]);
    }
#pragma unroll
    for (int s = 0; s < OZ_NS; ++s)
      *reinterpret_cast<uint4*>(out0 + oz_off(s * BMAX + k, j0)) = *reinterpret_cast<const uint4*>(out[s]);
  }
}

// ----------------------------------------------------------- the product
// One 128-row tile: out[r * nk + k] (+)= (A X)[r][k] for r < m, k < nk, with A
// given as NSA slices per K chunk (block (c, s) at Sg + (c * NSA + s) * OZ_AB),
// its row exponents erow[r], the X chunk blocks at Xg and the column
// exponents fcol[k].  OZ_THREADS threads, OZ_SMEM bytes of dynamic shared
// memory.  A with fewer slices than X (NSA < OZ_NS, e.g. FP32 data, exact in 5)
// pairs every A slice with the X slices t <= OZ_NS - 1 - s as before.
template <int NSA>
__device__ __forceinline__ void oz_tile(const __nv_bfloat16* __restrict__ Sg, int nch,
                                        const __nv_bfloat16* __restrict__ Xg, const int* __restrict__ erow,
                                        const int* __restrict__ fcol, double* __restrict__ out, int m, int nk,
                                        bool add, int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char oz_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(oz_raw) + 1023) & ~uintptr_t(1023));
  __nv_bfloat16* sB = reinterpret_cast<__nv_bfloat16*>(smem);  // [2][OZ_BB]
  __nv_bfloat16* sA = sB + 2 * OZ_BB;                          // [OZ_ASTAGES][OZ_AB]
  __shared__ __align__(8) uint64_t bar_a[OZ_ASTAGES], bar_afree[OZ_ASTAGES], bar_b[2], bar_bfree[2], bar_done;
  __shared__ uint32_t tmem_base;
  __shared__ volatile int abort_flag;
  __shared__ long long a_issued, b_issued, mma_groups;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    for (int s = 0; s < OZ_ASTAGES; ++s) { mbar_init(&bar_a[s], 1); mbar_init(&bar_afree[s], 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(&bar_b[b], 1); mbar_init(&bar_bfree[b], 1); }
    mbar_init(&bar_done, 1);
    abort_flag = 0;
    a_issued = b_issued = mma_groups = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(512));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (warp == 4) {
    // ------------------------------------------------ copies (one thread)
    if (lane == 0) {
      long long g = 0;
      for (int c = 0; c < nch && !abort_flag; ++c) {
        const int bb = c & 1;
        if (c >= 2 && !mbar_wait(&bar_bfree[bb], (uint32_t)(((c - 2) >> 1) & 1))) { abort_flag = 1; break; }
        mbar_expect_tx(&bar_b[bb], OZ_BB * 2);
        bulk_g2s(sB + bb * OZ_BB, Xg + (long long)c * OZ_BB, OZ_BB * 2, &bar_b[bb]);
        b_issued = c + 1;
        for (int s = 0; s < NSA; ++s, ++g) {
          const int st = (int)(g % OZ_ASTAGES);
          if (g >= OZ_ASTAGES &&
              !mbar_wait(&bar_afree[st], (uint32_t)(((g - OZ_ASTAGES) / OZ_ASTAGES) & 1))) { abort_flag = 1; break; }
          mbar_expect_tx(&bar_a[st], OZ_AB * 2);
          bulk_g2s(sA + st * OZ_AB, Sg + ((long long)c * NSA + s) * OZ_AB, OZ_AB * 2, &bar_a[st]);
          a_issued = g + 1;
        }
      }
    }
  } else if (warp == 5) {
    // ------------------------------------------------ MMAs (one thread)
    if (lane == 0) {
      long long g = 0;
      for (int c = 0; c < nch && !abort_flag; ++c) {
        const int bb = c & 1;
        if (!mbar_wait(&bar_b[bb], (uint32_t)((c >> 1) & 1))) { abort_flag = 1; break; }
        const uint32_t b0 = smem_u32(sB + bb * OZ_BB);
        for (int s = 0; s < NSA; ++s, ++g) {
          const int st = (int)(g % OZ_ASTAGES);
          if (!mbar_wait(&bar_a[st], (uint32_t)((g / OZ_ASTAGES) & 1))) { abort_flag = 1; break; }
          tc_fence_after();
          const uint32_t a0 = smem_u32(sA + st * OZ_AB);
          const int nt = OZ_NS - s;  // X slices t = 0 .. nt-1 pair with A slice s (s + t <= 7)
#pragma unroll
          for (int k16 = 0; k16 < OZ_KC / 16; ++k16) {
            const uint32_t koff = k16 * 2 * TC_LBO;
            const uint32_t acc = (c > 0 || k16 > 0 || s > 0) ? 1u : 0u;
            // t = 0..3 -> D_{s+t} at TMEM column 64 (s + t), N = 64 min(nt, 4)
            const int n1 = min(nt, 4);
            mma_bf16(tmem + (uint32_t)(s * BMAX), tc_desc(a0 + koff), tc_desc(b0 + koff),
                     oz_idesc(OZ_M, n1 * BMAX), acc);
            if (nt > 4)
              mma_bf16(tmem + (uint32_t)((s + 4) * BMAX), tc_desc(a0 + koff),
                       tc_desc(b0 + koff + (uint32_t)(4 * BMAX / 8) * TC_SBO), oz_idesc(OZ_M, (nt - 4) * BMAX), acc);
          }
          mma_commit(&bar_afree[st]);
          mma_groups = g + 1;
        }
        if (abort_flag) break;
        mma_commit(&bar_bfree[bb]);
      }
      mma_commit(&bar_done);
    }
  } else {
    // ------------------------------------------------ epilogue (128 threads)
    const int r = warp * 32 + lane;  // TMEM lane = tile row
    const uint32_t trow = (uint32_t)(warp * 32) << 16;
    if (mbar_wait(&bar_done, 0u) && !abort_flag) {
      tc_fence_after();
      const int e = r < m ? erow[r] : 0;
#pragma unroll 1
      for (int cg = 0; cg < BMAX / 16; ++cg) {
        float sh[16], sl2[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) { sh[i] = 0.f; sl2[i] = 0.f; }
#pragma unroll 1
        for (int dd = OZ_NS - 1; dd >= 0; --dd) {  // smallest terms first
          float v[16];
          tmem_ld16(tmem + trow + (uint32_t)(dd * BMAX + cg * 16), v);
          const float sc = ldexpf(1.f, -6 * (dd + 2));
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            float t, er;
            two_sum(sh[i], v[i] * sc, t, er);
            sh[i] = t;
            sl2[i] += er;
          }
        }
        if (r < m) {
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int k = cg * 16 + i;
            if (k < nk) {
              const double v = ldexp((double)sh[i] + (double)sl2[i], e + fcol[k]);
              double* o = out + (long long)r * nk + k;
              *o = add ? *o + v : v;
            }
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
    const long long ga = a_issued, gb = b_issued, gm = mma_groups;
    if (gm > 0) mbar_wait(&bar_afree[(gm - 1) % OZ_ASTAGES], (uint32_t)(((gm - 1) / OZ_ASTAGES) & 1));
    for (long long q = gm; q < ga; ++q) mbar_wait(&bar_a[q % OZ_ASTAGES], (uint32_t)((q / OZ_ASTAGES) & 1));
    for (long long q = gb - 2 > 0 ? gb - 2 : 0; q < gb; ++q) mbar_wait(&bar_b[q & 1], (uint32_t)((q >> 1) & 1));
    atomicOr(err, DE_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512));
}

// yrep[rep + r][k] = (S X)[r][k] for the rows of one 128-row tile of one
// subdomain; grid (max row tiles, nsub), OZ_THREADS threads, OZ_SMEM bytes.
__global__ void __launch_bounds__(OZ_THREADS, 1)
    kb_schur_oz(const DevSub* __restrict__ ds, const __nv_bfloat16* __restrict__ sl,
                const long long* __restrict__ soff, const long long* __restrict__ eoff, const int* __restrict__ erow,
                const __nv_bfloat16* __restrict__ xl, const long long* __restrict__ xoff, const int* __restrict__ fcol,
                double* __restrict__ yrep, int nk, int* __restrict__ err, const int* __restrict__ ndone) {
  if (batch_all_done(ndone, nk)) return;
  const DevSub d = ds[blockIdx.y];
  const int rt = blockIdx.x, r0 = rt * OZ_M;
  if (r0 >= d.ni) return;
  const int nch = (d.ni + OZ_KC - 1) / OZ_KC;
  oz_tile<OZ_NS>(sl + soff[blockIdx.y] + (long long)rt * nch * OZ_NS * OZ_AB, nch, xl + xoff[blockIdx.y],
                 erow + eoff[blockIdx.y] + r0, fcol + blockIdx.y * BMAX, yrep + (long long)(d.rep + r0) * nk,
                 min(OZ_M, d.ni - r0), nk, false, err);
}

// ------------------------------------------- FP32 matrices (preconditioner)
// Exact products of the FP32 preconditioner blocks Z, Phi and Phi^T with the
// FP64 vectors: the blocks are cut into OZ_NA slices and the vectors into
// OZ_NS slices as for the Schur apply.  Every application is then the same
// linear operator, without the rounding noise of FP32 products that delays the
// outer PCG on ill-conditioned problems.  The slices of a row are scaled by
// the row's largest entry, so seven 6-bit slices hold every FP32 entry down to
// 2^-43 of it: a fixed (and almost symmetric) change of the blocks of at most
// ni 2^-44 of the row's scale in a product.  Fewer slices leave a larger
// asymmetric change: at 48^3 three-level elasticity with stiff inclusions the
// batched mixed columns took +9 iterations over the oracle with five slices,
// +5 with six and +3 with seven or eight.
constexpr int OZ_NA = 7;

// one sliced matrix: rows m, K range k, row-major FP32 source at src with
// leading dimension ld; slice blocks at soff, row exponents at eoff
struct OzMat {
  long long src, soff, eoff;
  int ld, m, k;
};

// erow[eoff + r] for r < m rounded up to the 128-row tile (padding rows 0);
// warp per row, grid (rows / 8, matrices)
__global__ void kb_oz_row_exp_a(const OzMat* __restrict__ mats, const float* __restrict__ pool,
                                int* __restrict__ erow) {
  const OzMat a = mats[blockIdx.y];
  const int r = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (r >= (a.m + OZ_M - 1) / OZ_M * OZ_M) return;
  float mx = 0.f;
  if (r < a.m)
    for (int j = lane; j < a.k; j += 32) mx = fmaxf(mx, fabsf(pool[a.src + (long long)r * a.ld + j]));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) erow[a.eoff + r] = oz_exp((double)mx);
}

// slice blocks ((rt * nch + c) * OZ_NA + s) * OZ_AB from soff; grid (tiles x chunks, matrices)
__global__ void __launch_bounds__(256) kb_oz_slice_a(const OzMat* __restrict__ mats, const float* __restrict__ pool,
                                                     const int* __restrict__ erow, __nv_bfloat16* __restrict__ sl) {
  const OzMat a = mats[blockIdx.y];
  const int nch = (a.k + OZ_KC - 1) / OZ_KC, nrt = (a.m + OZ_M - 1) / OZ_M;
  if ((int)blockIdx.x >= nch * nrt) return;
  const int rt = blockIdx.x / nch, c = blockIdx.x % nch;
  __nv_bfloat16* base = sl + a.soff + ((long long)rt * nch + c) * OZ_NA * OZ_AB;
  for (int task = threadIdx.x; task < OZ_M * (OZ_KC / 8); task += 256) {
    const int r = task / (OZ_KC / 8), k0 = (task % (OZ_KC / 8)) * 8;
    const int gr = rt * OZ_M + r;
    const float sc = ldexpf(1.f, -erow[a.eoff + gr]);
    __align__(16) __nv_bfloat16 out[OZ_NA][8];
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
      const int gk = c * OZ_KC + k0 + kk;
      const float v = (gr < a.m && gk < a.k) ? pool[a.src + (long long)gr * a.ld + gk] : 0.f;
      float q[OZ_NA];
      oz_split(v * sc, 0.f, q);
#pragma unroll
      for (int s = 0; s < OZ_NA; ++s) out[s][kk] = __float2bfloat16_rn(q[s]);
    }
#pragma unroll
    for (int s = 0; s < OZ_NA; ++s)
      *reinterpret_cast<uint4*>(base + (long long)s * OZ_AB + oz_off(r, k0)) = *reinterpret_cast<const uint4*>(out[s]);
  }
}

// one output tile of a sliced product
struct OzJob {
  long long a;    // first slice block of the tile's first K chunk (bf16 elements)
  long long e;    // row exponent of tile row 0
  long long x;    // first X chunk block (bf16 elements)
  long long out;  // output row of tile row 0 (rows of nk doubles)
  int f;          // column exponents at fcol + f
  int m, nch;     // valid rows (<= OZ_M), K chunks (>= 1)
  int add;        // 1: added to the output
};

// grid: one CTA per job; OZ_THREADS threads, OZ_SMEM bytes
__global__ void __launch_bounds__(OZ_THREADS, 1)
    kb_gemm_oz(const OzJob* __restrict__ jobs, const __nv_bfloat16* __restrict__ sl, const int* __restrict__ erow,
               const __nv_bfloat16* __restrict__ xl, const int* __restrict__ fcol, double* __restrict__ out, int nk,
               int* __restrict__ err, const int* __restrict__ ndone) {
  if (batch_all_done(ndone, nk)) return;
  const OzJob j = jobs[blockIdx.x];
  oz_tile<OZ_NA>(sl + j.a, j.nch, xl + j.x, erow + j.e, fcol + j.f, out + j.out * nk, j.m, nk, j.add != 0, err);
}

}  // namespace bddc
