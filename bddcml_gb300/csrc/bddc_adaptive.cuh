// Adaptive face constraints on the GPU: batched LOBPCG over all face pairs
// (the reference runs one BLOPEX LOBPCG per pair, lobpcg_driver.c:169-304,
// with the operators of adaptivity_mvecmult, module_adaptivity.f90:2560-3023).
//
// For pair p (subdomains i, j; n = ni + nj interface dofs of both) the pencil is
//   A = P (I-E)^T S (I-E) P,   B = P S P,   S = diag(S_i, S_j),
// P the orthogonal projection onto null([C_i -C_j]) (P = I - Q Q^T), E the
// weighted average on the dofs both subdomains share, and the largest k <= 10
// eigenpairs are sought.  The preconditioner is P diag(Z_i, Z_j) P with the
// subdomain corrections Z of the current BDDC preconditioner (the local part of
// the reference's pair BDDC, idoper 5).
//
// Data: one arena of vector blocks; block b of pair p holds n x KMAX values,
// column c, row r at arena[b * nvec + vo + c * n + r].  The S and Z products run
// per subdomain over all the pair columns that subdomain takes part in (one
// read of S_s per product): S in FP64 (the float2 pair hi + lo), the
// preconditioner Z in FP32; everything else is FP64, including the
// Rayleigh-Ritz step (SVQB + Jacobi, one warp per pair).
#pragma once

#include <cuda_runtime.h>

#include "bddc_setup_kernels.cuh"

namespace bddc {

constexpr int AD_KM = 10;     // eigenvectors per pair at most (AdaptivePairs::KMAX)
constexpr int AD_MAXM = 48;   // columns of Q at most
constexpr int AD_NB = 3 * AD_KM;
enum { AB_X = 0, AB_AX, AB_BX, AB_W, AB_AW, AB_BW, AB_Y, AB_AY, AB_BY, AB_T1, AB_T2, AB_NBLK };

struct PairDev {
  int si, sj, ni, n, m, k, cbeg, cend;
  long long vo, qo;
};

// columns of one batched product: per subdomain s the entries [ptr[s], ptr[s+1]),
// each an input and an output column offset in the arena (ni_s rows)
struct ColTab {
  const int* ptr;
  const long long* in;
  const long long* out;
};

__device__ __forceinline__ double ad_uniform(unsigned long long x) {
  // splitmix64 finaliser -> (-1, 1)
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  x ^= x >> 31;
  return (double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

// X = random (seeded by pair, column, row)
__global__ void k_ad_random(const PairDev* __restrict__ pd, double* __restrict__ va, long long nvec) {
  const PairDev q = pd[blockIdx.x];
  double* X = va + AB_X * nvec + q.vo;
  for (int c = 0; c < q.k; ++c)
    for (int r = threadIdx.x; r < q.n; r += blockDim.x)
      X[(long long)c * q.n + r] = ad_uniform(((unsigned long long)blockIdx.x << 36) ^ ((unsigned long long)c << 28) ^ r);
}

// V <- V - Q (Q^T V) on block b0 (and b1 if >= 0): grid (npair, 1 or 2)
__global__ void __launch_bounds__(256) k_ad_project(const PairDev* __restrict__ pd, const double* __restrict__ Q,
                                                    double* __restrict__ va, long long nvec, int b0, int b1) {
  const PairDev q = pd[blockIdx.x];
  if (q.k == 0 || q.m == 0) return;
  double* V = va + (blockIdx.y == 0 ? b0 : b1) * nvec + q.vo;
  const double* Qp = Q + q.qo;
  __shared__ double t[AD_MAXM][AD_KM];
  __shared__ double red[8][AD_KM];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j = 0; j < q.m; ++j) {
    double acc[AD_KM];
#pragma unroll
    for (int c = 0; c < AD_KM; ++c) acc[c] = 0.0;
    for (int r = threadIdx.x; r < q.n; r += blockDim.x) {
      const double qr = Qp[(long long)j * q.n + r];
#pragma unroll
      for (int c = 0; c < AD_KM; ++c)
        if (c < q.k) acc[c] += qr * V[(long long)c * q.n + r];
    }
#pragma unroll
    for (int c = 0; c < AD_KM; ++c) {
      double v = acc[c];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) red[wid][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < q.k) {
      double v = 0.0;
      for (int w = 0; w < 8; ++w) v += red[w][threadIdx.x];
      t[j][threadIdx.x] = v;
    }
    __syncthreads();
  }
  for (int r = threadIdx.x; r < q.n; r += blockDim.x) {
    double acc[AD_KM];
#pragma unroll
    for (int c = 0; c < AD_KM; ++c) acc[c] = 0.0;
    for (int j = 0; j < q.m; ++j) {
      const double qr = Qp[(long long)j * q.n + r];
#pragma unroll
      for (int c = 0; c < AD_KM; ++c) acc[c] += qr * t[j][c];
    }
    for (int c = 0; c < q.k; ++c) V[(long long)c * q.n + r] -= acc[c];
  }
}

// out = (I - E) in, or (I - E)^T in (adaptivity_apply_weights / _R / _RT,
// module_adaptivity.f90:3097-3184): zero except on the shared dofs
__global__ void __launch_bounds__(256) k_ad_ire(const PairDev* __restrict__ pd, const int* __restrict__ ca,
                                                const int* __restrict__ cb, const double* __restrict__ wa,
                                                const double* __restrict__ wb, double* __restrict__ va,
                                                long long nvec, int bin, int bout, int transpose) {
  const PairDev q = pd[blockIdx.x];
  if (q.k == 0) return;
  const double* in = va + bin * nvec + q.vo;
  double* out = va + bout * nvec + q.vo;
  for (long long e = threadIdx.x; e < (long long)q.k * q.n; e += blockDim.x) out[e] = 0.0;
  __syncthreads();
  for (int e = q.cbeg + threadIdx.x; e < q.cend; e += blockDim.x) {
    const int a = ca[e], b = cb[e];
    const double xa0 = wa[e], xb0 = wb[e];
    for (int c = 0; c < q.k; ++c) {
      const double xa = in[(long long)c * q.n + a], xb = in[(long long)c * q.n + b];
      if (!transpose) {
        const double avg = xa0 * xa + xb0 * xb;
        out[(long long)c * q.n + a] = xa - avg;
        out[(long long)c * q.n + b] = xb - avg;
      } else {
        const double sm = xa + xb;
        out[(long long)c * q.n + a] = xa - xa0 * sm;
        out[(long long)c * q.n + b] = xb - xb0 * sm;
      }
    }
  }
}

// matrix entry in the compute type CT: a float2 (hi, lo) pair is the value
// hi + lo (FP64 compute) or hi (FP32 compute)
template <typename CT, typename MT>
__device__ __forceinline__ CT ad_mval(const MT* p) { return (CT)(*p); }
template <>
__device__ __forceinline__ float ad_mval<float, float2>(const float2* p) { return p->x; }
template <>
__device__ __forceinline__ double ad_mval<double, float2>(const float2* p) {
  return (double)p->x + (double)p->y;
}

// Batched products out_col = M_s in_col over the columns of a ColTab, M_s the
// subdomain's S (USE_Z false) or Z (USE_Z true), NI x NI, symmetric.  Tile of
// 64 rows x 64 columns per CTA, K in chunks of 32 staged in shared memory,
// multiply-add in CT: FP64 for S (the small eigenvalues of the face pencils
// sit far below FP32 rounding of S in high-contrast problems), FP32 for the
// preconditioner Z.  Grid (ceil(maxNI / 64), ceil(maxcols / 64), nsub).
template <typename MT, bool USE_Z, typename CT>
__global__ void __launch_bounds__(256) k_ad_gemm(const DevSub* __restrict__ ds, const MT* __restrict__ Mpool,
                                                 ColTab tab, double* __restrict__ va) {
  const int s = blockIdx.z;
  const DevSub d = ds[s];
  const int r0 = blockIdx.x * 64;
  const int cbeg = tab.ptr[s], ncol = tab.ptr[s + 1] - cbeg;
  const int c0 = blockIdx.y * 64;
  if (r0 >= d.ni || c0 >= ncol) return;
  const MT* M = Mpool + (USE_Z ? d.oZ : d.oS);
  __shared__ CT As[32][64 + 2];
  __shared__ CT Bs[32][64 + 2];
  __shared__ long long inoff[64], outoff[64];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  if (tid < 64) {
    const bool ok = c0 + tid < ncol;
    inoff[tid] = ok ? tab.in[cbeg + c0 + tid] : -1;
    outoff[tid] = ok ? tab.out[cbeg + c0 + tid] : -1;
  }
  CT acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = CT(0);
  __syncthreads();
  for (int k0 = 0; k0 < d.ni; k0 += 32) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = tid + 256 * i;
      const int row = e >> 5, kk = e & 31;
      const int gr = r0 + row, gk = k0 + kk;
      As[kk][row] = (gr < d.ni && gk < d.ni) ? ad_mval<CT, MT>(M + (long long)gr * d.NI + gk) : CT(0);
      const long long io = inoff[row];  // row doubles as the column index of the B tile
      Bs[kk][row] = (io >= 0 && gk < d.ni) ? (CT)va[io + gk] : CT(0);
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; ++kk) {
      CT a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gr = r0 + ty * 4 + i;
    if (gr >= d.ni) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const long long oo = outoff[tx * 4 + j];
      if (oo >= 0) va[oo + gr] = (double)acc[i][j];
    }
  }
}

// The same batched product with S as the float2 pair hi + lo in double-float
// arithmetic on the FP32 pipes (df_mac, bddc_df.cuh).

__global__ void __launch_bounds__(256) k_ad_gemm_df(const DevSub* __restrict__ ds, const float2* __restrict__ Spool,
                                                    ColTab tab, double* __restrict__ va) {
  const int s = blockIdx.z;
  const DevSub d = ds[s];
  const int r0 = blockIdx.x * 64;
  const int cbeg = tab.ptr[s], ncol = tab.ptr[s + 1] - cbeg;
  const int c0 = blockIdx.y * 64;
  if (r0 >= d.ni || c0 >= ncol) return;
  const float2* M = Spool + d.oS;
  __shared__ float Ah[32][64 + 4], Al[32][64 + 4], Bh[32][64 + 4], Bl[32][64 + 4];
  __shared__ long long inoff[64], outoff[64];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  if (tid < 64) {
    const bool ok = c0 + tid < ncol;
    inoff[tid] = ok ? tab.in[cbeg + c0 + tid] : -1;
    outoff[tid] = ok ? tab.out[cbeg + c0 + tid] : -1;
  }
  float sh[4][4], sl[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) { sh[i][j] = 0.f; sl[i][j] = 0.f; }
  __syncthreads();
  for (int k0 = 0; k0 < d.ni; k0 += 32) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int e = tid + 256 * i;
      const int row = e >> 5, kk = e & 31;
      const int gr = r0 + row, gk = k0 + kk;
      float2 a = make_float2(0.f, 0.f);
      if (gr < d.ni && gk < d.ni) a = M[(long long)gr * d.NI + gk];
      Ah[kk][row] = a.x;
      Al[kk][row] = a.y;
      const long long io = inoff[row];  // row doubles as the column index of the B tile
      const double x = (io >= 0 && gk < d.ni) ? va[io + gk] : 0.0;
      const float xh = (float)x;
      Bh[kk][row] = xh;
      Bl[kk][row] = (float)(x - (double)xh);
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < 32; ++kk) {
      float ah[4], al[4], bh[4], bl[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) { ah[i] = Ah[kk][ty * 4 + i]; al[i] = Al[kk][ty * 4 + i]; }
#pragma unroll
      for (int j = 0; j < 4; ++j) { bh[j] = Bh[kk][tx * 4 + j]; bl[j] = Bl[kk][tx * 4 + j]; }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) df_mac(sh[i][j], sl[i][j], ah[i], al[i], bh[j], bl[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gr = r0 + ty * 4 + i;
    if (gr >= d.ni) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const long long oo = outoff[tx * 4 + j];
      if (oo >= 0) va[oo + gr] = (double)sh[i][j] + (double)sl[i][j];
    }
  }
}

// Gram blocks G_{A,B}[u][v] = basis_u^T image_v for u <= v < nb (basis X, W, Y;
// images AX.. or BX..), k x k each, into G[p][which][NB][NB].
// Grid (npair, 6, 2).
__global__ void __launch_bounds__(256) k_ad_gram(const PairDev* __restrict__ pd, const double* __restrict__ va,
                                                 long long nvec, double* __restrict__ G, int nb) {
  const PairDev q = pd[blockIdx.x];
  const int uv[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
  const int u = uv[blockIdx.y][0], v = uv[blockIdx.y][1];
  if (q.k == 0 || v >= nb) return;
  const int which = blockIdx.z;  // 0 A, 1 B
  const int basis[3] = {AB_X, AB_W, AB_Y};
  const int imgA[3] = {AB_AX, AB_AW, AB_AY};
  const int imgB[3] = {AB_BX, AB_BW, AB_BY};
  const double* U = va + basis[u] * nvec + q.vo;
  const double* V = va + (which == 0 ? imgA[v] : imgB[v]) * nvec + q.vo;
  __shared__ double su[AD_KM][33], sv[AD_KM][33];
  const int kk = q.k;
  const int i = threadIdx.x / AD_KM, j = threadIdx.x % AD_KM;
  const bool act = threadIdx.x < AD_KM * AD_KM && i < kk && j < kk;
  double acc = 0.0;
  for (int r0 = 0; r0 < q.n; r0 += 32) {
    for (int e = threadIdx.x; e < 32 * AD_KM; e += blockDim.x) {
      const int c = e >> 5, rr = e & 31;
      const bool ok = c < kk && r0 + rr < q.n;
      su[c][rr] = ok ? U[(long long)c * q.n + r0 + rr] : 0.0;
      sv[c][rr] = ok ? V[(long long)c * q.n + r0 + rr] : 0.0;
    }
    __syncthreads();
    if (act)
#pragma unroll 8
      for (int rr = 0; rr < 32; ++rr) acc += su[i][rr] * sv[j][rr];
    __syncthreads();
  }
  if (act) {
    double* Gp = G + ((long long)blockIdx.x * 2 + which) * AD_NB * AD_NB;
    const int gr = u * kk + i, gc = v * kk + j;
    Gp[gr * AD_NB + gc] = acc;
    if (u != v) Gp[gc * AD_NB + gr] = acc;
  }
}

// cyclic Jacobi eigen-decomposition of the symmetric nn x nn matrix a (in
// shared memory, leading dimension 33) by one warp; z receives the eigenvectors
// (columns), the eigenvalues are left on the diagonal of a
__device__ void ad_jacobi(double (*a)[33], double (*z)[33], int nn) {
  const int lane = threadIdx.x & 31;
  for (int r = 0; r < nn; ++r)
    if (lane < nn) z[r][lane] = (r == lane) ? 1.0 : 0.0;
  __syncwarp();
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = 0.0, dg = 0.0;
    for (int r = 0; r < nn; ++r)
      if (lane < nn) {
        if (lane != r) off += a[r][lane] * a[r][lane];
        else dg += a[r][r] * a[r][r];
      }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      dg += __shfl_xor_sync(0xffffffffu, dg, o);
    }
    if (off <= 1e-28 * dg || off == 0.0) break;
    for (int p = 0; p < nn - 1; ++p)
      for (int q = p + 1; q < nn; ++q) {
        // rotation computed by lane 0 (FP64 divide and square roots are slow
        // on this part) and broadcast; rotations of negligible entries skipped
        double c = 1.0, s = 0.0;
        int skip = 1;
        if (lane == 0) {
          const double apq = a[p][q], app = a[p][p], aqq = a[q][q];
          if (fabs(apq) > 1e-16 * sqrt(fabs(app * aqq)) && apq != 0.0) {
            const double th = (aqq - app) / (2.0 * apq);
            const double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
            c = 1.0 / sqrt(t * t + 1.0);
            s = t * c;
            skip = 0;
          }
        }
        skip = __shfl_sync(0xffffffffu, skip, 0);
        if (skip) continue;
        c = __shfl_sync(0xffffffffu, c, 0);
        s = __shfl_sync(0xffffffffu, s, 0);
        __syncwarp();
        if (lane < nn) {
          const double xp = a[p][lane], xq = a[q][lane];
          a[p][lane] = c * xp - s * xq;
          a[q][lane] = s * xp + c * xq;
        }
        __syncwarp();
        if (lane < nn) {
          const double xp = a[lane][p], xq = a[lane][q];
          a[lane][p] = c * xp - s * xq;
          a[lane][q] = s * xp + c * xq;
          const double zp = z[lane][p], zq = z[lane][q];
          z[lane][p] = c * zp - s * zq;
          z[lane][q] = s * zp + c * zq;
        }
        __syncwarp();
        if (lane == 0) { a[p][q] = 0.0; a[q][p] = 0.0; }
        __syncwarp();
      }
  }
}

// Rayleigh-Ritz on span(basis), nb blocks of k columns: SVQB on G_B (scaled
// to unit diagonal, directions below 1e-8 of the largest dropped: below that
// the Gram entries are at the noise level of the S products), then the
// largest k eigenpairs of V^T G_A V.  C (nb k x k, row-major in C[p]) maps the
// basis to the new X; lam receives the Ritz values (descending).  One warp per pair.
__global__ void __launch_bounds__(32) k_ad_rr(const PairDev* __restrict__ pd, const double* __restrict__ G,
                                              double* __restrict__ C, double* __restrict__ lam, int nb) {
  const PairDev q = pd[blockIdx.x];
  if (q.k == 0) return;
  const int k = q.k, nn = nb * k, lane = threadIdx.x;
  __shared__ double a[32][33], z[32][33], v[32][33], ga[32][33];
  __shared__ double dsc[32];
  __shared__ int keep[32];
  __shared__ int nkeep;
  const double* GA = G + ((long long)blockIdx.x * 2 + 0) * AD_NB * AD_NB;
  const double* GB = G + ((long long)blockIdx.x * 2 + 1) * AD_NB * AD_NB;
  for (int r = 0; r < nn; ++r)
    if (lane < nn) {
      ga[r][lane] = 0.5 * (GA[r * AD_NB + lane] + GA[lane * AD_NB + r]);
      a[r][lane] = 0.5 * (GB[r * AD_NB + lane] + GB[lane * AD_NB + r]);
    }
  __syncwarp();
  if (lane < nn) dsc[lane] = a[lane][lane] > 0.0 ? 1.0 / sqrt(a[lane][lane]) : 0.0;
  __syncwarp();
  for (int r = 0; r < nn; ++r)
    if (lane < nn) a[r][lane] *= dsc[r] * dsc[lane];
  __syncwarp();
  ad_jacobi(a, z, nn);
  // keep the directions with sigma > 1e-8 max sigma
  if (lane == 0) {
    double smax = 0.0;
    for (int r = 0; r < nn; ++r) smax = fmax(smax, a[r][r]);
    int cnt = 0;
    for (int r = 0; r < nn; ++r)
      if (a[r][r] > 1e-8 * smax && smax > 0.0) keep[cnt++] = r;
    nkeep = cnt;
  }
  __syncwarp();
  const int nk = nkeep;
  // v = D z_keep sigma^-1/2  (nn x nk)
  for (int r = 0; r < nn; ++r)
    if (lane < nk) v[r][lane] = dsc[r] * z[r][keep[lane]] / sqrt(a[keep[lane]][keep[lane]]);
  __syncwarp();
  // a = v^T ga v (nk x nk): first z = ga v (nn x nk)
  for (int r = 0; r < nn; ++r)
    if (lane < nk) {
      double t = 0.0;
      for (int c = 0; c < nn; ++c) t += ga[r][c] * v[c][lane];
      z[r][lane] = t;
    }
  __syncwarp();
  for (int r = 0; r < nk; ++r)
    if (lane < nk) {
      double t = 0.0;
      for (int c = 0; c < nn; ++c) t += v[c][r] * z[c][lane];
      a[r][lane] = t;
    }
  __syncwarp();
  for (int r = 0; r < nk; ++r)
    if (lane < nk && lane > r) {
      const double m = 0.5 * (a[r][lane] + a[lane][r]);
      a[r][lane] = m;
      a[lane][r] = m;
    }
  __syncwarp();
  ad_jacobi(a, z, nk);
  // order: descending Ritz values
  if (lane == 0) {
    for (int r = 0; r < nk; ++r) keep[r] = r;
    for (int r = 0; r < nk; ++r)
      for (int c = r + 1; c < nk; ++c)
        if (a[keep[c]][keep[c]] > a[keep[r]][keep[r]]) { const int t = keep[r]; keep[r] = keep[c]; keep[c] = t; }
  }
  __syncwarp();
  double* Cp = C + (long long)blockIdx.x * AD_NB * AD_KM;
  for (int c = 0; c < k; ++c) {
    if (c < nk) {
      if (lane < nn) {
        double t = 0.0;
        for (int j = 0; j < nk; ++j) t += v[lane][j] * z[j][keep[c]];
        Cp[lane * AD_KM + c] = t;
      }
      if (lane == 0) lam[(long long)blockIdx.x * AD_KM + c] = a[keep[c]][keep[c]];
    } else if (lane < nn) {  // fewer independent directions than wanted: keep the old column
      Cp[lane * AD_KM + c] = lane == c ? 1.0 : 0.0;
    }
  }
}

// X <- [X W Y] C, Y <- [W Y] C(k:, :) for the triple t (0: X,W,Y; 1: AX,AW,AY;
// 2: BX,BW,BY), row by row in place.  Grid (npair, 3, row blocks of 128).
__global__ void __launch_bounds__(128) k_ad_update(const PairDev* __restrict__ pd, double* __restrict__ va,
                                                   long long nvec, const double* __restrict__ C, int nb) {
  const PairDev q = pd[blockIdx.x];
  if (q.k == 0) return;
  const int k = q.k, nn = nb * k;
  __shared__ double cs[AD_NB][AD_KM];
  const double* Cp = C + (long long)blockIdx.x * AD_NB * AD_KM;
  for (int e = threadIdx.x; e < nn * AD_KM; e += blockDim.x) cs[e / AD_KM][e % AD_KM] = Cp[e];
  __syncthreads();
  const int r = blockIdx.z * blockDim.x + threadIdx.x;
  if (r >= q.n) return;
  const int tb[3][3] = {{AB_X, AB_W, AB_Y}, {AB_AX, AB_AW, AB_AY}, {AB_BX, AB_BW, AB_BY}};
  const int t = blockIdx.y;
  double* B0 = va + tb[t][0] * nvec + q.vo;
  double* B1 = va + tb[t][1] * nvec + q.vo;
  double* B2 = va + tb[t][2] * nvec + q.vo;
  double in[AD_NB];
  for (int c = 0; c < k; ++c) {
    in[c] = B0[(long long)c * q.n + r];
    if (nb > 1) in[k + c] = B1[(long long)c * q.n + r];
    if (nb > 2) in[2 * k + c] = B2[(long long)c * q.n + r];
  }
  for (int c = 0; c < k; ++c) {
    double x = 0.0, y = 0.0;
    for (int j = 0; j < k; ++j) x += in[j] * cs[j][c];
    for (int j = k; j < nn; ++j) y += in[j] * cs[j][c];
    B0[(long long)c * q.n + r] = x + y;
    if (nb > 1) B2[(long long)c * q.n + r] = y;
  }
}

// Coarse correction of the pair preconditioner (the coarse part of the
// reference's pair BDDC, adaptivity_mvecmult idoper 5, module_adaptivity.f90:
// 2760-2890): W += Phi K^+ Phi^T R with Phi = diag(Phi_i, Phi_j) and K the
// pair's assembled local coarse matrices (regularised along the null space
// of S, which the projection removes).  R in block T1, W in block W.
// Grid (npair, KMAX), 256 threads.
constexpr int AD_NUMAX = 256;
struct PairCoarse {
  const int* nu;          // coarse dofs of the pair (union of both subdomains')
  const int* mofs;        // offset of the pair's maps: nc_i entries, then nc_j
  const int* map;         // local coarse dof -> pair coarse dof
  const long long* kofs;  // offset of the pair's K^+ (nu x nu, row-major)
  const double* kinv;
};
template <typename T>
__global__ void __launch_bounds__(256) k_ad_coarse(const PairDev* __restrict__ pd, PairCoarse pc,
                                                   const DevSub* __restrict__ ds, const T* __restrict__ pcpool,
                                                   double* __restrict__ va, long long nvec) {
  const PairDev q = pd[blockIdx.x];
  const int c = blockIdx.y;
  if (c >= q.k) return;
  const int nu = pc.nu[blockIdx.x];
  __shared__ double rc[AD_NUMAX], u[AD_NUMAX];
  for (int i = threadIdx.x; i < nu; i += blockDim.x) rc[i] = 0.0;
  __syncthreads();
  const double* R = va + AB_T1 * nvec + q.vo + (long long)c * q.n;
  double* W = va + AB_W * nvec + q.vo + (long long)c * q.n;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int* mp = pc.map + pc.mofs[blockIdx.x];
  for (int side = 0; side < 2; ++side) {
    const DevSub d = ds[side == 0 ? q.si : q.sj];
    const int roff = side == 0 ? 0 : q.ni;
    const int* ms = mp + (side == 0 ? 0 : ds[q.si].nc);
    const T* phi = pcpool + d.oPhi;
    for (int qq = wid; qq < d.nc; qq += 8) {
      double t = 0.0;
      for (int r = lane; r < d.ni; r += 32) t += (double)phi[(long long)r * d.ncp + qq] * R[roff + r];
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (lane == 0) atomicAdd(&rc[ms[qq]], t);
    }
  }
  __syncthreads();
  const double* K = pc.kinv + pc.kofs[blockIdx.x];
  for (int i = threadIdx.x; i < nu; i += blockDim.x) {
    double t = 0.0;
    for (int j = 0; j < nu; ++j) t += K[(long long)i * nu + j] * rc[j];
    u[i] = t;
  }
  __syncthreads();
  for (int side = 0; side < 2; ++side) {
    const DevSub d = ds[side == 0 ? q.si : q.sj];
    const int roff = side == 0 ? 0 : q.ni;
    const int* ms = mp + (side == 0 ? 0 : ds[q.si].nc);
    const T* phi = pcpool + d.oPhi;
    for (int r = threadIdx.x; r < d.ni; r += blockDim.x) {
      double t = 0.0;
      for (int qq = 0; qq < d.nc; ++qq) t += (double)phi[(long long)r * d.ncp + qq] * u[ms[qq]];
      W[roff + r] += t;
    }
  }
}

// R = A X - B X diag(lam) into block T1
__global__ void k_ad_residual(const PairDev* __restrict__ pd, double* __restrict__ va, long long nvec,
                              const double* __restrict__ lam) {
  const PairDev q = pd[blockIdx.x];
  const int r = blockIdx.y * blockDim.x + threadIdx.x;
  if (r >= q.n) return;
  for (int c = 0; c < q.k; ++c) {
    const long long o = q.vo + (long long)c * q.n + r;
    va[AB_T1 * nvec + o] = va[AB_AX * nvec + o] - lam[(long long)blockIdx.x * AD_KM + c] * va[AB_BX * nvec + o];
  }
}

// relative residual ||A x - lam B x|| / ||A x|| of every Ritz pair
__global__ void __launch_bounds__(256) k_ad_resnorm(const PairDev* __restrict__ pd, const double* __restrict__ va,
                                                    long long nvec, const double* __restrict__ lam,
                                                    double* __restrict__ out) {
  const PairDev q = pd[blockIdx.x];
  const int c = blockIdx.y;
  if (c >= q.k) return;
  __shared__ double red[2][8];
  double rr = 0.0, aa = 0.0;
  const double l = lam[(long long)blockIdx.x * AD_KM + c];
  for (int r = threadIdx.x; r < q.n; r += blockDim.x) {
    const long long o = q.vo + (long long)c * q.n + r;
    const double ax = va[AB_AX * nvec + o];
    const double res = ax - l * va[AB_BX * nvec + o];
    rr += res * res;
    aa += ax * ax;
  }
  for (int o = 16; o > 0; o >>= 1) {
    rr += __shfl_xor_sync(0xffffffffu, rr, o);
    aa += __shfl_xor_sync(0xffffffffu, aa, o);
  }
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = rr; red[1][threadIdx.x >> 5] = aa; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r2 = 0.0, a2 = 0.0;
    for (int w = 0; w < 8; ++w) { r2 += red[0][w]; a2 += red[1][w]; }
    out[(long long)blockIdx.x * AD_KM + c] = a2 > 0.0 ? sqrt(r2 / a2) : 0.0;
  }
}

// gather n-long arena columns (offsets src) into a packed buffer (offsets dst)
__global__ void k_ad_gather(const double* __restrict__ va, const long long* __restrict__ src,
                            const long long* __restrict__ dst, const int* __restrict__ len, double* __restrict__ out) {
  const int c = blockIdx.x;
  for (int r = threadIdx.x; r < len[c]; r += blockDim.x) out[dst[c] + r] = va[src[c] + r];
}

}  // namespace bddc
