// Kernels of the batched interface PCG: nk right-hand sides of one assembled
// problem advanced together, each with its own PCG recurrence (scalars, stop
// test, Lanczos coefficients), so that every column follows the iteration of
// krylov_bddcpcg (module_krylov.f90:545-888) for its own load.
//
// Layout: every batched vector is dof-major with the columns interleaved,
// v[g * nk + k], nk a power of two <= 64.  A gather of one interface dof then
// moves all columns in one coalesced segment, and the per-subdomain applies
// (Schur operator, local preconditioner with the coarse correction, interior
// resolve) become GEMMs that read each subdomain matrix once per iteration for
// all columns instead of once per column.
#pragma once

#include "bddc_pcg_kernels.cuh"

namespace bddc {

constexpr int BMAX = 64;  // columns per batch: one GEMM column tile
constexpr int GM = 64;    // GEMM rows per CTA
constexpr int GK = 32;    // GEMM K chunk

// One product of a batched GEMM:  out = addend + A1 B1 + A2 B2  (rows m).
// A1 is m x k1 (row stride lda), A2 m x k2 (row stride lda2, optional);
// B1 / B2 are row blocks of the B buffers starting at rows ob / ob2; the
// result rows start at oo.  For double-float planes oA2 is the low plane.
struct GemmDesc {
  long long oA, oA2;
  long long ob, ob2;
  long long oo;
  int m, k1, k2, lda, lda2, pad;
};

__device__ __forceinline__ bool batch_all_done(const int* ndone, int nk) { return ndone && *ndone >= nk; }

// --------------------------------------------------------------- gathers
// b[j][k] = split(sign * x[uniq[j]][k]) for replicated interface index j
__global__ void kb_gather_df(long long nrep, int lg, const int* __restrict__ uniq, double sign,
                             const double* __restrict__ x, float2* __restrict__ b, const int* __restrict__ ndone,
                             const double* __restrict__ w = nullptr) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (nrep << lg)) return;
  const long long j = e >> lg;
  const int k = (int)(e & (nk - 1));
  double t = sign * x[((long long)uniq[j] << lg) + k];
  if (w) t *= w[j];
  const dfloat v = df_from_double(t);
  b[e] = make_float2(v.hi, v.lo);
}

// b[e] = split(x[e]) for cnt entries (the batched operands of the double-float products)
__global__ void kb_to_df(long long cnt, const double* __restrict__ x, float2* __restrict__ b,
                         const int* __restrict__ ndone, int nk) {
  if (batch_all_done(ndone, nk)) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= cnt) return;
  const dfloat v = df_from_double(x[e]);
  b[e] = make_float2(v.hi, v.lo);
}

// a matrix pool of n doubles as two float planes: hi at [0, n), lo at [n, 2n)
__global__ void kb_to_planes(long long n, const double* __restrict__ x, float* __restrict__ p) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const dfloat v = df_from_double(x[e]);
  p[e] = v.hi;
  p[n + e] = v.lo;
}

// b[j][k] = T(sign * w[j] * x[uniq[j]][k])  (w optional)
template <typename T>
__global__ void kb_gather_t(long long nrep, int lg, const int* __restrict__ uniq, const double* __restrict__ w,
                            double sign, const double* __restrict__ x, T* __restrict__ b,
                            const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (nrep << lg)) return;
  const long long j = e >> lg;
  const int k = (int)(e & (nk - 1));
  double v = sign * x[((long long)uniq[j] << lg) + k];
  if (w) v *= w[j];
  b[e] = T(v);
}

// ---------------------------------------------------------------- GEMMs
// Double-float product with FP64-class accuracy on the FP32 pipes (A stored as
// (hi, lo) pairs, interleaved float2 or two planes; B pre-split float2):
//   out[oo + r][c] = addend + sum_j A[r][j] B[ob + j][c],   c < nk.
// 256 threads, 64 x 64 output tile, each thread rows ty + 16 i, columns
// tx + 16 j (conflict-free shared-memory reads).
template <bool PLANES>
__global__ void __launch_bounds__(256) kb_gemm_df(const GemmDesc* __restrict__ gd, const float* __restrict__ A,
                                                  const float2* __restrict__ B, int ldb, double* out,
                                                  const double* addend, int ldo, int nk,
                                                  const int* __restrict__ ndone) {
  if (batch_all_done(ndone, nk)) return;
  const GemmDesc d = gd[blockIdx.y];
  const int r0 = blockIdx.x * GM;
  if (r0 >= d.m) return;
  __shared__ float Ah[GK][GM + 1], Al[GK][GM + 1], Bh[GK][BMAX], Bl[GK][BMAX];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  float sh[4][4], sl[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) { sh[i][j] = 0.f; sl[i][j] = 0.f; }
  for (int k0 = 0; k0 < d.k1; k0 += GK) {
    if (!PLANES) {  // float2 pairs, two consecutive columns per 16-byte load
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int e = tid + 256 * i;
        const int row = e >> 4, m2 = e & 15;
        const int gr = r0 + row, gk = k0 + 2 * m2;
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
        if (gr < d.m && gk < d.k1) {
          a = __ldg(reinterpret_cast<const float4*>(A + 2 * (d.oA + (long long)gr * d.lda + gk)));
          if (gk + 1 >= d.k1) { a.z = 0.f; a.w = 0.f; }
        }
        Ah[2 * m2][row] = a.x;
        Al[2 * m2][row] = a.y;
        Ah[2 * m2 + 1][row] = a.z;
        Al[2 * m2 + 1][row] = a.w;
      }
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int e = tid + 256 * i;
        const int row = e >> 5, kk = e & 31;
        const int gr = r0 + row, gk = k0 + kk;
        float h = 0.f, l = 0.f;
        if (gr < d.m && gk < d.k1) {
          const long long o = (long long)gr * d.lda + gk;
          h = __ldg(A + d.oA + o);
          l = __ldg(A + d.oA2 + o);
        }
        Ah[kk][row] = h;
        Al[kk][row] = l;
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = tid + 256 * i;
      const int kk = e >> 6, c = e & 63;
      const int gk = k0 + kk;
      float2 b = make_float2(0.f, 0.f);
      if (gk < d.k1 && c < nk) b = B[(d.ob + gk) * ldb + c];
      Bh[kk][c] = b.x;
      Bl[kk][c] = b.y;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < GK; ++kk) {
      float ah[4], al[4], bh[4], bl[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) { ah[i] = Ah[kk][ty + 16 * i]; al[i] = Al[kk][ty + 16 * i]; }
#pragma unroll
      for (int j = 0; j < 4; ++j) { bh[j] = Bh[kk][tx + 16 * j]; bl[j] = Bl[kk][tx + 16 * j]; }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) df_mac(sh[i][j], sl[i][j], ah[i], al[i], bh[j], bl[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gr = r0 + ty + 16 * i;
    if (gr >= d.m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = tx + 16 * j;
      if (c >= nk) continue;
      const long long o = (d.oo + gr) * ldo + c;
      const double v = (double)sh[i][j] + (double)sl[i][j];
      out[o] = addend ? addend[o] + v : v;
    }
  }
}

// Product in the working precision T with T accumulation, two K segments:
//   out[oo + r][c] = addend + sum_j A1[r][j] B1[ob + j][c] + sum_j A2[r][j] B2[ob2 + j][c]
// BM x 64 output tile per CTA (256 threads, rows ty + 16 i, columns tx + 16 j),
// K chunks of 32 streamed through a STAGES-deep cp.async ring so that the
// operand loads of later chunks are in flight while a chunk is multiplied.
// FP32 uses 128-row tiles; FP64 (a small fraction of the FP32 rate on this
// part, and used for the small level-2 problem) 32-row tiles, for more CTAs.
// Requires nk % 4 == 0 and 16-byte aligned rows (row strides and offsets
// multiples of 16 / sizeof(T) elements); partial chunks are zero-filled.
template <typename T>
struct GtCfg {
  static constexpr int BM = sizeof(T) == 4 ? 128 : 32;
  static constexpr int RI = BM / 16;  // rows per thread
  static constexpr int STAGES = sizeof(T) == 4 ? 4 : 3;
  static constexpr int VEC = 16 / sizeof(T);  // elements per 16-byte copy
  static constexpr int LDA = GK + VEC;        // padded row stride of the A tile
  static constexpr int A_ELEMS = BM * LDA;
  static constexpr int B_ELEMS = GK * BMAX;
  static constexpr size_t SMEM = (size_t)STAGES * (A_ELEMS + B_ELEMS) * sizeof(T);
};

__device__ __forceinline__ void cp_async16(void* dst, const void* src, int bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(
                   static_cast<unsigned>(__cvta_generic_to_shared(dst))),
               "l"(src), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <typename T>
__global__ void __launch_bounds__(256) kb_gemm_t(const GemmDesc* __restrict__ gd, const T* __restrict__ A,
                                                 const T* __restrict__ B1, const T* __restrict__ B2, int ldb,
                                                 double* out, const double* addend, int ldo, int nk,
                                                 const int* __restrict__ ndone) {
  using C = GtCfg<T>;
  if (batch_all_done(ndone, nk)) return;
  const GemmDesc d = gd[blockIdx.y];
  const int r0 = blockIdx.x * C::BM;
  if (r0 >= d.m) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* As = reinterpret_cast<T*>(smraw);
  T* Bs = As + C::STAGES * C::A_ELEMS;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int n1 = (d.k1 + GK - 1) / GK, nch = n1 + (d.k2 + GK - 1) / GK;
  auto load = [&](int c) {
    const int buf = c % C::STAGES;
    const bool seg1 = c < n1;
    const int kb = seg1 ? c * GK : (c - n1) * GK;
    const int K = seg1 ? d.k1 : d.k2;
    const T* Ab = A + (seg1 ? d.oA : d.oA2);
    const int lda = seg1 ? d.lda : d.lda2;
    const T* Bb = seg1 ? B1 + d.ob * ldb : B2 + d.ob2 * ldb;
    T* as = As + buf * C::A_ELEMS;
    T* bs = Bs + buf * C::B_ELEMS;
    constexpr int CPR = GK / C::VEC;  // 16-byte copies per A row
#pragma unroll
    for (int q = 0; q < C::BM * CPR / 256; ++q) {
      const int e = tid + 256 * q;
      const int row = e / CPR, kc = (e % CPR) * C::VEC;
      const int gr = r0 + row, gk = kb + kc;
      const int nb = (gr < d.m && gk < K) ? min(C::VEC, K - gk) * (int)sizeof(T) : 0;
      const T* src = nb ? Ab + (long long)gr * lda + gk : Ab;
      cp_async16(as + row * C::LDA + kc, src, nb);
    }
    constexpr int CPB = BMAX / C::VEC;  // 16-byte copies per B row
#pragma unroll
    for (int q = 0; q < GK * CPB / 256; ++q) {
      const int e = tid + 256 * q;
      const int row = e / CPB, cc = (e % CPB) * C::VEC;
      const int gk = kb + row;
      const int nb = (gk < K && cc < nk) ? 16 : 0;
      const T* src = nb ? Bb + (long long)gk * ldb + cc : Bb;
      cp_async16(bs + row * BMAX + cc, src, nb);
    }
  };
  T acc[C::RI][4];
#pragma unroll
  for (int i = 0; i < C::RI; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
#pragma unroll
  for (int st = 0; st < C::STAGES - 1; ++st) {
    if (st < nch) load(st);
    cp_async_commit();
  }
  for (int c = 0; c < nch; ++c) {
    cp_async_wait<C::STAGES - 2>();
    __syncthreads();
    if (c + C::STAGES - 1 < nch) load(c + C::STAGES - 1);
    cp_async_commit();
    const T* as = As + (c % C::STAGES) * C::A_ELEMS;
    const T* bs = Bs + (c % C::STAGES) * C::B_ELEMS;
#pragma unroll 4
    for (int kk = 0; kk < GK; ++kk) {
      T a[C::RI], b[4];
#pragma unroll
      for (int i = 0; i < C::RI; ++i) a[i] = as[(ty + 16 * i) * C::LDA + kk];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = bs[kk * BMAX + tx + 16 * j];
#pragma unroll
      for (int i = 0; i < C::RI; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
    }
  }
  cp_async_wait<0>();
#pragma unroll
  for (int i = 0; i < C::RI; ++i) {
    const int gr = r0 + ty + 16 * i;
    if (gr >= d.m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = tx + 16 * j;
      if (c >= nk) continue;
      const long long o = (d.oo + gr) * ldo + c;
      const double v = (double)acc[i][j];
      out[o] = addend ? addend[o] + v : v;
    }
  }
}

// ------------------------------------------------- preconditioner pieces
// coarse residual of each subdomain, rcs[coff + c][k] = sum_i Phi[i][c] aux[rep + i][k]
// (dd_phisi_dual_apply, module_dd.f90:6126-6206); grid (nsub, ceil(ncpmax / 32))
template <typename T>
__global__ void __launch_bounds__(256) kb_phit(const DevSub* __restrict__ ds, const T* __restrict__ pcpool,
                                               const T* __restrict__ aux, int lg, double* __restrict__ rcs,
                                               const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const DevSub s = ds[blockIdx.x];
  const int c0 = blockIdx.y * 32;
  if (c0 >= s.nc) return;
  __shared__ T as[32][BMAX];
  __shared__ T ps[32][33];
  const int tid = threadIdx.x, k = tid & (nk - 1), cl = tid >> lg, ncl = 256 >> lg;
  T acc[8];
#pragma unroll
  for (int m = 0; m < 8; ++m) acc[m] = T(0);
  for (int i0 = 0; i0 < s.ni; i0 += 32) {
    for (int e = tid; e < 32 * nk; e += 256) {
      const int ii = e >> lg, kk = e & (nk - 1);
      as[ii][kk] = i0 + ii < s.ni ? aux[((long long)(s.rep + i0 + ii) << lg) + kk] : T(0);
    }
    for (int e = tid; e < 32 * 32; e += 256) {
      const int ii = e >> 5, cc = e & 31;
      ps[ii][cc] = (i0 + ii < s.ni && c0 + cc < s.nc) ? pcpool[s.oPhi + (long long)(i0 + ii) * s.ncp + c0 + cc] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int c = cl + ncl * m;
      if (c < 32)
        for (int ii = 0; ii < 32; ++ii) acc[m] += ps[ii][c] * as[ii][k];
    }
    __syncthreads();
  }
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const int c = cl + ncl * m;
    if (c < 32 && c0 + c < s.nc) rcs[((long long)(s.coff + c0 + c) << lg) + k] = (double)acc[m];
  }
}

// Phi^T of every subdomain (ncp x NI row-major at oT[s], padding zero), the
// operand of the coarse-residual product rcs = Phi^T W r
template <typename T>
__global__ void kb_phi_transpose(const DevSub* __restrict__ ds, const T* __restrict__ pcpool,
                                 const long long* __restrict__ oT, T* __restrict__ phit) {
  const DevSub s = ds[blockIdx.y];
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)s.ncp * s.NI) return;
  const int c = (int)(e / s.NI), i = (int)(e % s.NI);
  phit[oT[blockIdx.y] + e] = (c < s.nc && i < s.ni) ? pcpool[s.oPhi + (long long)i * s.ncp + c] : T(0);
}

// rc[q][k] = sum over the subdomain constraints mapped to coarse dof q (and
// over the nparts partial planes of rcs, pstride apart, of a split-K product)
__global__ void kb_coarse_gather(int ndofc, int lg, const int* __restrict__ cptr, const int* __restrict__ csub,
                                 const int* __restrict__ cloc, const DevSub* __restrict__ ds,
                                 const double* __restrict__ rcs, double* __restrict__ rc,
                                 const int* __restrict__ ndone, int nparts = 1, long long pstride = 0) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ((long long)ndofc << lg)) return;
  const int q = (int)(e >> lg), k = (int)(e & (nk - 1));
  double t = 0.0;
  for (int p = cptr[q]; p < cptr[q + 1]; ++p) {
    const long long o = ((long long)(ds[csub[p]].coff + cloc[p]) << lg) + k;
    for (int h = 0; h < nparts; ++h) t += rcs[o + h * pstride];
  }
  rc[e] = t;
}

// ucs[e][k] = T(uc[cmap[e]][k]): the coarse solution at each subdomain constraint
template <typename T>
__global__ void kb_gather_uc(long long ncon, int lg, const int* __restrict__ cmap, const double* __restrict__ uc,
                             T* __restrict__ ucs, const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (ncon << lg)) return;
  ucs[e] = T(uc[((long long)cmap[e >> lg] << lg) + (e & (nk - 1))]);
}

template <typename T>
__global__ void kb_to_t(long long cnt, const double* __restrict__ v, T* __restrict__ out, int nk,
                        const int* __restrict__ ndone) {
  if (batch_all_done(ndone, nk)) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < cnt) out[e] = T(v[e]);
}

// res = rc - Ac uc with the sparse FP64 coarse matrix
__global__ void kb_coarse_res(int n, int lg, const int* __restrict__ ptr, const int* __restrict__ col,
                              const double* __restrict__ val, const double* __restrict__ rc,
                              const double* __restrict__ uc, double* __restrict__ res, const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ((long long)n << lg)) return;
  const int i = (int)(e >> lg), k = (int)(e & (nk - 1));
  double t = rc[e];
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) t -= val[q] * uc[((long long)col[q] << lg) + k];
  res[e] = t;
}

// ------------------------------------------------ assembly and reductions
// per-column block sums of the threads' partials (thread t holds column t % nk)
__device__ __forceinline__ void col_partials(double v, int nk, double* sh, double* __restrict__ part, int npart) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int st = RT / 2; st >= nk; st >>= 1) {
    if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
    __syncthreads();
  }
  if (threadIdx.x < nk) part[(long long)threadIdx.x * npart + blockIdx.x] = sh[threadIdx.x];
}

// out[g][k] = sum of the subdomain rows (zero at fixed dofs if asked);
// partial (p, out)_w per column when p is given
__global__ void __launch_bounds__(RT) kb_assemble_dot(int n, int lg, Owners own, const double* __restrict__ yrep,
                                                      const int* __restrict__ fixed, const double* __restrict__ wsum,
                                                      const double* __restrict__ p, double* __restrict__ out,
                                                      double* __restrict__ part, int npart, int zero_fixed,
                                                      const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  __shared__ double sh[RT];
  const int k = threadIdx.x & (nk - 1), rl = threadIdx.x >> lg, nrl = RT >> lg;
  double loc = 0.0;
  for (long long g = (long long)blockIdx.x * nrl + rl; g < n; g += (long long)gridDim.x * nrl) {
    double v = 0.0;
    for (int q = own.ptr[g]; q < own.ptr[g + 1]; ++q) v += yrep[((long long)own.rep[q] << lg) + k];
    if (zero_fixed && fixed && fixed[g]) v = 0.0;
    const long long e = (g << lg) + k;
    out[e] = v;
    if (p) loc += wsum[g] * p[e] * v;
  }
  if (part) col_partials(loc, nk, sh, part, npart);
}

// z[g][k] = sum_s w_s zrep_s (the coarse correction is already in zrep); partial (r, z)_w
__global__ void __launch_bounds__(RT) kb_assemble_z(int n, int lg, Owners own, const double* __restrict__ zrep,
                                                    const double* __restrict__ wrep, const double* __restrict__ wsum,
                                                    const double* __restrict__ r, double* __restrict__ z,
                                                    double* __restrict__ part, int npart,
                                                    const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  __shared__ double sh[RT];
  const int k = threadIdx.x & (nk - 1), rl = threadIdx.x >> lg, nrl = RT >> lg;
  double loc = 0.0;
  for (long long g = (long long)blockIdx.x * nrl + rl; g < n; g += (long long)gridDim.x * nrl) {
    double v = 0.0;
    for (int q = own.ptr[g]; q < own.ptr[g + 1]; ++q) {
      const int j = own.rep[q];
      v += wrep[j] * zrep[((long long)j << lg) + k];
    }
    const long long e = (g << lg) + k;
    z[e] = v;
    loc += wsum[g] * r[e] * v;
  }
  if (part) col_partials(loc, nk, sh, part, npart);
}

// partial (a, b)_w per column
__global__ void __launch_bounds__(RT) kb_dot(int n, int lg, const double* __restrict__ a, const double* __restrict__ b,
                                             const double* __restrict__ wsum, double* __restrict__ part, int npart) {
  const int nk = 1 << lg;
  __shared__ double sh[RT];
  const int k = threadIdx.x & (nk - 1), rl = threadIdx.x >> lg, nrl = RT >> lg;
  double loc = 0.0;
  for (long long g = (long long)blockIdx.x * nrl + rl; g < n; g += (long long)gridDim.x * nrl) {
    const long long e = (g << lg) + k;
    loc += wsum[g] * a[e] * b[e];
  }
  col_partials(loc, nk, sh, part, npart);
}

__global__ void kb_axpy(long long cnt, double a, const double* __restrict__ x, double* __restrict__ y) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < cnt) y[e] += a * x[e];
}

// x[g][k] = x0[g] for every column
__global__ void kb_bcast(int n, int lg, const double* __restrict__ x0, double* __restrict__ x) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < ((long long)n << lg)) x[e] = x0[e >> lg];
}

// ------------------------------------------- multi-column interior solves
// Blocks V of NO rows x vld columns per subdomain at voff (row-major); the
// right-hand sides are interleaved rows (fo_off + r) x nk.
template <typename T>
__global__ void kb_v_fill(const DevSub* __restrict__ ds, int lg, const double* __restrict__ rhs,
                          const long long* __restrict__ fo_off, const long long* __restrict__ voff, int vld,
                          T* __restrict__ v) {
  const int nk = 1 << lg;
  const DevSub s = ds[blockIdx.y];
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)s.NO * vld) return;
  const int r = (int)(e / vld), k = (int)(e % vld);
  v[voff[blockIdx.y] + e] = (r < s.no && k < nk) ? T(rhs[((fo_off[blockIdx.y] + r) << lg) + k]) : T(0);
}

// component outc = F - A_oo (X0 [+ D1]) with FP64-accurate double-float sums,
// stored as FP32 (the refinement residuals of the mixed-precision solves);
// grid (ceil(maxNO / 8), nsub), vld threads (one per column), 8 rows per CTA
__global__ void kb_v_residual(const DevSub* __restrict__ ds, CsrView koo, int lg, const double* __restrict__ rhs,
                              const long long* __restrict__ fo_off, const long long* __restrict__ voff, int vld,
                              float* __restrict__ v, int xpair, int outc) {
  const int nk = 1 << lg;
  const DevSub s = ds[blockIdx.y];
  const int k = threadIdx.x;
  const long long comp = (long long)s.NO * vld;
  const float* X0 = v + voff[blockIdx.y];
  const float* X1 = X0 + comp;
  float* out = v + voff[blockIdx.y] + outc * comp;
  const int* p = koo.ptr + s.koo;
  for (int r = blockIdx.x * 8; r < min(s.NO, blockIdx.x * 8 + 8); ++r) {
    float res = 0.f;
    if (r < s.no && k < nk) {
      dfacc acc;
      acc.add_df(df_from_double(rhs[((fo_off[blockIdx.y] + r) << lg) + k]));
      for (int q = p[r]; q < p[r + 1]; ++q) {
        const long long o = (long long)koo.col[q] * vld + k;
        const dfloat a = df_from_double(-koo.val[q]);
        if (xpair) acc.fma_df(a, dfloat{X0[o], X1[o]});
        else acc.fma_df(a, X0[o]);
      }
      res = acc.value().hi;
    }
    out[(long long)r * vld + k] = res;
  }
}

// value of the interior solution V[r][k]: the FP32 pair (X0, D1) or the FP64 block
__device__ __forceinline__ double v_value(const float* v, long long comp, long long o) {
  return (double)v[o] + (double)v[comp + o];
}
__device__ __forceinline__ double v_value(const double* v, long long, long long o) { return v[o]; }

// grep[rep + i][k] = f_i - A_io V  (module_dd.f90:6995-7257), double-float sums
template <typename T>
__global__ void kb_v_grep(const DevSub* __restrict__ ds, CsrView kio, int lg, const double* __restrict__ fi,
                          const long long* __restrict__ voff, int vld, const T* __restrict__ v,
                          double* __restrict__ grep) {
  const int nk = 1 << lg;
  const DevSub s = ds[blockIdx.y];
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ((long long)s.ni << lg)) return;
  const int i = (int)(e >> lg), k = (int)(e & (nk - 1));
  const long long o = ((long long)(s.rep + i) << lg) + k;
  const T* V = v + voff[blockIdx.y];
  const long long comp = (long long)s.NO * vld;
  dfacc acc;
  acc.add_df(df_from_double(fi[o]));
  const int* p = kio.ptr + s.kio;
  for (int q = p[i]; q < p[i + 1]; ++q)
    acc.fma_df(df_from_double(-kio.val[q]), df_from_double(v_value(V, comp, (long long)kio.col[q] * vld + k)));
  grep[o] = acc.to_double();
}

// vo[uo_off + r][k] = V[r][k]
template <typename T>
__global__ void kb_v_out(const DevSub* __restrict__ ds, int lg, const long long* __restrict__ voff, int vld,
                         const T* __restrict__ v, const long long* __restrict__ uo_off, double* __restrict__ vo) {
  const int nk = 1 << lg;
  const DevSub s = ds[blockIdx.y];
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ((long long)s.no << lg)) return;
  const int r = (int)(e >> lg), k = (int)(e & (nk - 1));
  vo[((uo_off[blockIdx.y] + r) << lg) + k] = v_value(v + voff[blockIdx.y], (long long)s.NO * vld, (long long)r * vld + k);
}

// ---------------------------------------------------------------- scalars
// per column: normres0 = |r|, rmp = (r, z); columns past nrhs, with a zero
// reduced rhs or a zero initial residual stop at once
__global__ void kb_init(PcgCtl* __restrict__ ctl, const double* __restrict__ pgg, const double* __restrict__ prr,
                        const double* __restrict__ prz, int npart, double tol, int maxit, int ndecrmax, int nrhs,
                        int* __restrict__ ndone) {
  __shared__ double sh[32];
  const int k = blockIdx.x;
  const double gg = sum_parts(pgg + (long long)k * npart, npart, sh);
  const double rr = sum_parts(prr + (long long)k * npart, npart, sh);
  const double rz = sum_parts(prz + (long long)k * npart, npart, sh);
  if (threadIdx.x == 0) {
    PcgCtl c{};
    c.normres0 = sqrt(rr);
    c.rmp = rz;
    c.tol = tol;
    c.lastres = 1.0;
    c.iter = 1;
    c.maxit = maxit;
    c.ndecrmax = ndecrmax;
    if (k >= nrhs || gg == 0.0 || rr == 0.0) {
      c.done = 1;
      c.reason = 0;
      c.num_iter = 0;
      c.nw = 0;
      atomicAdd(ndone, 1);
    }
    ctl[k] = c;
  }
}

__global__ void kb_sc_alpha(PcgCtl* ctl, const double* __restrict__ part, int npart) {
  PcgCtl* c = ctl + blockIdx.x;
  if (c->done) return;
  __shared__ double sh[32];
  const double pap = sum_parts(part + (long long)blockIdx.x * npart, npart, sh);
  if (threadIdx.x == 0) {
    c->pap = pap;
    if (!(pap > 0.0)) c->warn |= 1;
    c->alpha = c->rmp / pap;
  }
}

__global__ void kb_sc_res(PcgCtl* ctl, const double* __restrict__ part, int npart, double* __restrict__ hist,
                          int ldh, int* __restrict__ ndone) {
  PcgCtl* c = ctl + blockIdx.x;
  if (c->done) return;
  __shared__ double sh[32];
  const double nr2 = sum_parts(part + (long long)blockIdx.x * npart, npart, sh);
  if (threadIdx.x == 0) {
    const int iter = c->iter;
    c->normres2 = nr2;
    const double relres = sqrt(nr2) / c->normres0;
    c->relres = relres;
    hist[(long long)blockIdx.x * ldh + iter - 1] = relres;
    int stop = 0;
    if (relres < c->tol) { stop = 1; c->reason = 0; }
    else if (iter == c->maxit) { stop = 1; c->reason = -1; }
    else {
      if (relres < c->lastres) c->ndecr = 0;
      else {
        c->ndecr += 1;
        if (c->ndecr >= c->ndecrmax) { stop = 1; c->reason = -2; }
      }
      c->lastres = relres;
    }
    if (stop) {
      c->done = 1;
      c->num_iter = iter;
      c->nw = iter - 1;
      atomicAdd(ndone, 1);
    }
  }
}

__global__ void kb_sc_beta(PcgCtl* ctl, const double* __restrict__ part, int npart, double* __restrict__ diag,
                           double* __restrict__ subdiag, int ldd) {
  PcgCtl* c = ctl + blockIdx.x;
  if (c->done) return;
  __shared__ double sh[32];
  const double rmp = sum_parts(part + (long long)blockIdx.x * npart, npart, sh);
  if (threadIdx.x == 0) {
    if (!(rmp > 0.0)) c->warn |= 2;
    const double beta = rmp / c->rmp;
    c->beta = beta;
    c->rmp = rmp;
    const int iter = c->iter;
    const double alpha = c->alpha;
    double* dg = diag + (long long)blockIdx.x * ldd;
    double* sd = subdiag + (long long)blockIdx.x * ldd;
    dg[iter - 1] += 1.0 / alpha;
    dg[iter] = beta / alpha;
    sd[iter - 1] = beta >= 0.0 ? -sqrt(beta) / alpha : 0.0;
    c->iter = iter + 1;
  }
}

// x += alpha p, r -= alpha ap for the running columns; partial (r, r)_w
__global__ void __launch_bounds__(RT) kb_update_xr(int n, int lg, const PcgCtl* __restrict__ ctl,
                                                   double* __restrict__ x, double* __restrict__ r,
                                                   const double* __restrict__ p, const double* __restrict__ ap,
                                                   const double* __restrict__ wsum, double* __restrict__ part,
                                                   int npart) {
  const int nk = 1 << lg;
  __shared__ double sh[RT];
  const int k = threadIdx.x & (nk - 1), rl = threadIdx.x >> lg, nrl = RT >> lg;
  const bool run = !ctl[k].done;
  const double alpha = ctl[k].alpha;
  double loc = 0.0;
  if (run)
    for (long long g = (long long)blockIdx.x * nrl + rl; g < n; g += (long long)gridDim.x * nrl) {
      const long long e = (g << lg) + k;
      x[e] += alpha * p[e];
      const double rv = r[e] - alpha * ap[e];
      r[e] = rv;
      loc += wsum[g] * rv * rv;
    }
  col_partials(loc, nk, sh, part, npart);
}

__global__ void kb_update_p(int n, int lg, const PcgCtl* __restrict__ ctl, double* __restrict__ p,
                            const double* __restrict__ z) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ((long long)n << lg)) return;
  const PcgCtl& c = ctl[e & ((1 << lg) - 1)];
  if (c.done) return;
  p[e] = z[e] + c.beta * p[e];
}

// ------------------------------------------------------------ three levels
// identity right-hand side of every band system (row-major, ld = ncol)
__global__ void k_band_identity(const BandDesc* __restrict__ bd, double* __restrict__ b) {
  const BandDesc d = bd[blockIdx.y];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < d.nb * NB && r < d.ncol) b[d.oB + (long long)r * d.ncol + r] = 1.0;
}

// level-2 interior loads fo[uo_off + r][k] = rc[mo[uo_off + r]][k]
__global__ void kb_l2_fo(int nfo, int lg, const int* __restrict__ mo, const double* __restrict__ rc,
                         double* __restrict__ fo, const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ((long long)nfo << lg)) return;
  fo[e] = rc[((long long)mo[e >> lg] << lg) + (e & (nk - 1))];
}

// fi[j][k] = w_j rc[mi[j]][k] on the level-2 interface (zero where unmapped)
__global__ void kb_l2_fi(int nrep, int lg, const int* __restrict__ mi, const double* __restrict__ wi,
                         const double* __restrict__ rc, double* __restrict__ fi, const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ((long long)nrep << lg)) return;
  const int j = (int)(e >> lg), k = (int)(e & (nk - 1));
  fi[e] = mi[j] >= 0 ? wi[j] * rc[((long long)mi[j] << lg) + k] : 0.0;
}

// grep = f_i - A_io v with v the interior solutions in the band block
__global__ void kb_reduced_rhs(const DevSub* __restrict__ ds, CsrView kio, int lg, const long long* __restrict__ rowoff,
                               const double* __restrict__ bb, const double* __restrict__ fi,
                               double* __restrict__ grep, const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const DevSub s = ds[blockIdx.y];
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ((long long)s.ni << lg)) return;
  const int i = (int)(e >> lg), k = (int)(e & (nk - 1));
  const long long o = ((long long)(s.rep + i) << lg) + k;
  double acc = fi[o];
  const int* p = kio.ptr + s.kio;
  const long long ro = rowoff[blockIdx.y];
  for (int q = p[i]; q < p[i + 1]; ++q) acc -= kio.val[q] * bb[(ro + kio.col[q]) * BMAX + k];
  grep[o] = acc;
}

// uc at the level-2 interior dofs (from the band block) and interface dofs (from z)
__global__ void kb_l2_out_o(const DevSub* __restrict__ ds, int lg, const long long* __restrict__ rowoff,
                            const long long* __restrict__ uo_off, const int* __restrict__ mo,
                            const double* __restrict__ bb, double* __restrict__ uc, const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const DevSub s = ds[blockIdx.y];
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ((long long)s.no << lg)) return;
  const int r = (int)(e >> lg), k = (int)(e & (nk - 1));
  uc[((long long)mo[uo_off[blockIdx.y] + r] << lg) + k] = bb[(rowoff[blockIdx.y] + r) * BMAX + k];
}

__global__ void kb_l2_out_i(int n, int lg, const int* __restrict__ mz, const double* __restrict__ z,
                            double* __restrict__ uc, const int* __restrict__ ndone) {
  const int nk = 1 << lg;
  if (batch_all_done(ndone, nk)) return;
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ((long long)n << lg)) return;
  uc[((long long)mz[e >> lg] << lg) + (e & (nk - 1))] = z[e];
}

}  // namespace bddc
