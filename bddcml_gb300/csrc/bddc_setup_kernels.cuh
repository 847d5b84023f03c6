// Setup kernels: block-band Cholesky, multi-RHS triangular solves, FP64-
// accurate Schur complements by refinement, constrained-Neumann
// preconditioner blocks and local coarse matrices.
//
// Reference counterparts (what is computed, not how):
//   interior factor A11 ............... module_dd.f90:4175-4295 (MUMPS there)
//   S = A22 - A21 A11^-1 A12 .......... module_dd.f90:6564-6699 (applied implicitly there)
//   [A C^T; C 0] factor ............... module_dd.f90:5211-5486 (MUMPS SYM=2 there)
//   coarse basis Phi, Ac = -lambda .... module_dd.f90:5489-5799
//   reduced rhs g = f2 - A21 A11^-1 f1  module_dd.f90:7138-7257
#pragma once

#include "bddc_df.cuh"
#include "bddc_kernels.cuh"

namespace bddc {

struct DevSub {
  int no, ni, nc, ncp;     // interior dofs, interface dofs, constraints, padded constraints
  int NO, NI, NR, NRC;     // padded: interior, interface, interior-RHS columns, Srho-RHS columns
  int nbo, w, nbi, nref;   // interior block rows, band blocks, interface block rows, refinement steps
  long long oL, oLinv;     // factor pool: interior band factor, inverted diagonal blocks
  long long oXc;           // factor pool: (nref+1) solution components, NO x NR each
  long long oLs, oLsinv;   // factor pool: preconditioner block factor
  long long oBs;           // factor pool: NI x NRC  [Srho^-1 | Y]
  long long oS;            // Schur pool: NI x NI
  long long oZ, oPhi;      // preconditioner pool: NI x NI, NI x ncp
  long long oGinv, oAc;    // small FP64 pool: ncp x ncp each
  int rep;                 // offset into replicated interface vectors
  int koo, koi, kio, kii;  // row-pointer offsets of the four CSR blocks
  int cptr;                // constraint row-pointer offset
  int coff;                // offset into per-constraint arrays (coarse map)
  double rho;              // penalty scale of the preconditioner block
  // general (nonsymmetric) matrices: the transposed upper LU factors (Ut) of the
  // interior and preconditioner blocks, the dual coarse basis input Y_dual and
  // the dual basis Phi_dual (oPhid = oPhi for symmetric matrices)
  long long oU, oUinv, oLsU, oLsUinv, oYd, oPhid;
};

// Cholesky factor and inverse of the 64 x 64 block in shared memory a (row
// stride NB + 1; its lower triangle, the factor L on exit) and L^-1 into inv
// (same stride, zero above the diagonal); NT = 256 threads.  Blocked in
// 16-column panels so that a block step needs 25 block barriers instead of
// the 320 of a column-by-column elimination:
//   factor, per panel: the 16 x 16 diagonal block by one warp with shuffles
//   (lane l owns row l), the rows below by forward substitution (a thread per
//   row), the trailing lower triangle by a rank-16 update;
//   inverse: the diagonal blocks' inverses column by column (warp p, lane j
//   owns column j of block p), then the blocks below the diagonal by distance,
//   Linv_pq = -Dinv_p sum_{m=q}^{p-1} L_pm Linv_mq.
// A non-positive or NaN pivot sets DE_PIVOT / DE_NAN in err and is replaced by 1.
template <typename T>
__device__ void diag_factor_inverse(T* a, T* inv, T* tmp, int* __restrict__ err) {
  constexpr int LD = NB + 1, PB = 16, NPB = NB / PB;
  static_assert(NT == PB * PB, "one thread per element of a 16 x 16 block");
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, tx = tid & 15, ty = tid >> 4;
  for (int p = 0; p < NPB; ++p) {
    const int c0 = p * PB;
    if (warp == 0) {
      T row[PB];
#pragma unroll
      for (int k = 0; k < PB; ++k) row[k] = lane < PB ? a[(c0 + lane) * LD + c0 + k] : T(0);
#pragma unroll
      for (int j = 0; j < PB; ++j) {
        T v = __shfl_sync(0xffffffffu, row[j], j);
        if (!(v > T(0))) {
          if (lane == 0) atomicOr(err, (v != v) ? DE_NAN : DE_PIVOT);
          v = T(1);
        }
        const T dj = sqrt(v);
        if (lane == j) row[j] = dj;
        else if (lane > j) row[j] /= dj;
#pragma unroll
        for (int kk = j + 1; kk < PB; ++kk) {
          const T lkj = __shfl_sync(0xffffffffu, row[j], kk);
          if (lane >= kk && lane < PB) row[kk] -= row[j] * lkj;
        }
      }
      if (lane < PB)
#pragma unroll
        for (int k = 0; k < PB; ++k)
          if (k <= lane) a[(c0 + lane) * LD + c0 + k] = row[k];
    }
    __syncthreads();
    for (int r = c0 + PB + tid; r < NB; r += NT) {  // rows below the diagonal block
      T x[PB];
#pragma unroll
      for (int c = 0; c < PB; ++c) {
        T t = a[r * LD + c0 + c];
#pragma unroll
        for (int k = 0; k < c; ++k) t -= x[k] * a[(c0 + c) * LD + c0 + k];
        x[c] = t / a[(c0 + c) * LD + c0 + c];
      }
#pragma unroll
      for (int c = 0; c < PB; ++c) a[r * LD + c0 + c] = x[c];
    }
    __syncthreads();
    for (int r = c0 + PB + ty; r < NB; r += PB)  // rank-16 update of the trailing lower triangle
      for (int q = c0 + PB + tx; q <= r; q += PB) {
        T t = a[r * LD + q];
#pragma unroll
        for (int k = 0; k < PB; ++k) t -= a[r * LD + c0 + k] * a[q * LD + c0 + k];
        a[r * LD + q] = t;
      }
    __syncthreads();
  }
  if (warp < NPB && lane < PB) {  // diagonal blocks of the inverse
    const int c0 = warp * PB, j = lane;
    T x[PB];
#pragma unroll
    for (int i = 0; i < PB; ++i) {
      T t = i == j ? T(1) : T(0);
#pragma unroll
      for (int k = 0; k < i; ++k) t -= a[(c0 + i) * LD + c0 + k] * x[k];
      x[i] = t / a[(c0 + i) * LD + c0 + i];
    }
#pragma unroll
    for (int i = 0; i < PB; ++i) inv[(c0 + i) * LD + c0 + j] = x[i];
  }
  for (int e = tid; e < NB * NB; e += NT) {
    const int r = e / NB, c = e % NB;
    if (c / PB > r / PB) inv[r * LD + c] = T(0);
  }
  __syncthreads();
  const int i = tid / PB, j = tid % PB;
  for (int dd = 1; dd < NPB; ++dd)
    for (int q = 0; q + dd < NPB; ++q) {
      const int p = q + dd;
      T t = T(0);
      for (int m = q; m < p; ++m)
#pragma unroll
        for (int k = 0; k < PB; ++k) t += a[(p * PB + i) * LD + m * PB + k] * inv[(m * PB + k) * LD + q * PB + j];
      tmp[i * (PB + 1) + j] = t;
      __syncthreads();
      T u = T(0);
      for (int k = 0; k <= i; ++k) u += inv[(p * PB + i) * LD + p * PB + k] * tmp[k * (PB + 1) + j];
      inv[(p * PB + i) * LD + q * PB + j] = -u;
      __syncthreads();
    }
}

// ------------------------------------------------------------ band factor
// Left-looking block Cholesky of a block-band matrix, step k:
//   diagonal: L_kk = chol(A_kk - sum_j L_kj L_kj^T), Linv_kk = L_kk^-1
//   below:    L_ik = (A_ik - sum_{j<k} L_ij L_kj^T) Linv_kk^T,  k < i <= k + w
// Shared memory of the diagonal step: a[NB][NB+1], inv[NB][NB+1], smA, smB.
template <typename T>
__device__ void chol_diag_step(const BandDesc& d, T* __restrict__ pool, int k, int* __restrict__ err, T* a, T* inv,
                               T* smA, T* smB, bool left = true) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
  tile_zero(acc);
  for (int j = left ? max(0, k - d.w) : k; j < k; ++j) {
    const T* Lkj = pool + band_block(d, k, j);
    tile_gemm<T, false, true>(acc, Lkj, NB, Lkj, NB, NB, smA, smB);
  }
  const T* Akk = pool + band_block(d, k, k);
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      int r = ty * 4 + q, c = tx * 4 + p;
      a[r * (NB + 1) + c] = Akk[r * NB + c] - acc[q][p];
    }
  __syncthreads();
  diag_factor_inverse<T>(a, inv, smA, err);
  T* Lkk = pool + band_block(d, k, k);
  T* Li = pool + d.oLinv + (long long)k * NB * NB;
  for (int e = tid; e < NB * NB; e += NT) {
    int r = e / NB, c = e % NB;
    Lkk[e] = c <= r ? a[r * (NB + 1) + c] : T(0);
    Li[e] = inv[r * (NB + 1) + c];
  }
}

template <typename T>
__device__ void chol_off_step(const BandDesc& d, T* __restrict__ pool, int k, int i, T* smA, T* smB) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
  tile_zero(acc);
  for (int j = max(0, i - d.w); j < k; ++j)
    tile_gemm<T, false, true>(acc, pool + band_block(d, i, j), NB, pool + band_block(d, k, j), NB, NB, smA, smB);
  T* Aik = pool + band_block(d, i, k);
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int p = 0; p < 4; ++p) Aik[(ty * 4 + q) * NB + tx * 4 + p] -= acc[q][p];
  __syncthreads();
  tile_zero(acc);
  tile_gemm<T, false, true>(acc, Aik, NB, pool + d.oLinv + (long long)k * NB * NB, NB, NB, smA, smB);
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int p = 0; p < 4; ++p) Aik[(ty * 4 + q) * NB + tx * 4 + p] = acc[q][p];
  __syncthreads();
}

// ------------------------------------------------------- band LU factor
// Left-looking block LU without pivoting of a general block-band matrix held
// in two lower block bands with the same shape: L (the diagonal block and the
// lower blocks of A on entry, the unit lower factor on exit) and Ut (the
// upper blocks of A transposed, Ut(i,k) = A(k,i)^T, on entry; U^T on exit).
// Step k:
//   diagonal: L_kk U_kk = A_kk - sum_{j<k} L_kj Ut_kj^T;  L_kk^-1 at L.oLinv, (U_kk^-1)^T at Ut.oLinv
//   below:    L_ik  = (A_ik  - sum_{j<k} L_ij  Ut_kj^T) Ut.inv_kk^T     (= ... U_kk^-1)
//             Ut_ik = (Ut_ik - sum_{j<k} Ut_ij L_kj^T)  L.inv_kk^T      (= (L_kk^-1 ...)^T)
// The forward solve with L then runs the Cholesky forward kernels on the L
// band, the backward solve with U the backward kernels on the Ut band (they
// apply Ut_kk^-T = U_kk^-1 and Ut_ik^T = U_ki).  The reference hands general
// matrices to MUMPS, which pivots (module_mumps.f90:443-511); block LU without
// pivoting needs diagonally dominant enough blocks, and a zero or non-finite
// pivot is reported in the error word.
template <typename T>
__device__ void lu_diag_step(const BandDesc& dl, const BandDesc& du, T* __restrict__ pool, int k,
                             int* __restrict__ err, T* a, T* inv, T* smA, T* smB) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
  tile_zero(acc);
  for (int j = max(0, k - dl.w); j < k; ++j)
    tile_gemm<T, false, true>(acc, pool + band_block(dl, k, j), NB, pool + band_block(du, k, j), NB, NB, smA, smB);
  const T* Akk = pool + band_block(dl, k, k);
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      int r = ty * 4 + q, c = tx * 4 + p;
      a[r * (NB + 1) + c] = Akk[r * NB + c] - acc[q][p];
    }
  __syncthreads();
  for (int c = 0; c < NB; ++c) {
    if (tid == 0) {
      T v = a[c * (NB + 1) + c];
      if (!(v == v) || v == T(0) || !(fabs((double)v) < 1e300)) {
        atomicOr(err, (v != v) ? DE_NAN : DE_PIVOT);
        a[c * (NB + 1) + c] = T(1);
      }
    }
    __syncthreads();
    const T dc = a[c * (NB + 1) + c];
    for (int r = c + 1 + tid; r < NB; r += NT) a[r * (NB + 1) + c] /= dc;
    __syncthreads();
    for (int r = c + 1 + ty; r < NB; r += 16) {  // trailing update of the whole block
      const T lr = a[r * (NB + 1) + c];
      for (int q = c + 1 + tx; q < NB; q += 16) a[r * (NB + 1) + q] -= lr * a[c * (NB + 1) + q];
    }
    __syncthreads();
  }
  // L_kk^-1 (unit lower) by elimination on the identity
  for (int e = tid; e < NB * NB; e += NT) {
    const int r = e / NB, c = e % NB;
    inv[r * (NB + 1) + c] = r == c ? T(1) : T(0);
  }
  __syncthreads();
  for (int kk = 0; kk < NB; ++kk) {
    for (int i = kk + 1 + ty; i < NB; i += 16) {
      const T lik = a[i * (NB + 1) + kk];
      for (int j = tx; j <= kk; j += 16) inv[i * (NB + 1) + j] -= lik * inv[kk * (NB + 1) + j];
    }
    __syncthreads();
  }
  T* Lkk = pool + band_block(dl, k, k);
  T* Li = pool + dl.oLinv + (long long)k * NB * NB;
  for (int e = tid; e < NB * NB; e += NT) {
    const int r = e / NB, c = e % NB;
    Lkk[e] = c < r ? a[r * (NB + 1) + c] : (c == r ? T(1) : T(0));
    Li[e] = inv[r * (NB + 1) + c];
  }
  __syncthreads();
  // U_kk^-1 (upper) by elimination on the identity from the last row up
  for (int e = tid; e < NB * NB; e += NT) {
    const int r = e / NB, c = e % NB;
    inv[r * (NB + 1) + c] = r == c ? T(1) : T(0);
  }
  __syncthreads();
  for (int kk = NB - 1; kk >= 0; --kk) {
    const T dk = a[kk * (NB + 1) + kk];
    for (int j = kk + tid; j < NB; j += NT) inv[kk * (NB + 1) + j] /= dk;
    __syncthreads();
    for (int i = ty; i < kk; i += 16) {
      const T uik = a[i * (NB + 1) + kk];
      for (int j = kk + tx; j < NB; j += 16) inv[i * (NB + 1) + j] -= uik * inv[kk * (NB + 1) + j];
    }
    __syncthreads();
  }
  T* Ukk = pool + band_block(du, k, k);
  T* Ui = pool + du.oLinv + (long long)k * NB * NB;
  for (int e = tid; e < NB * NB; e += NT) {
    const int r = e / NB, c = e % NB;  // transposed: (r, c) holds entry (c, r)
    Ukk[e] = c <= r ? a[c * (NB + 1) + r] : T(0);
    Ui[e] = inv[c * (NB + 1) + r];
  }
}

template <typename T>
__device__ void lu_off_step(const BandDesc& dl, const BandDesc& du, T* __restrict__ pool, int k, int i, T* smA,
                            T* smB) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  for (int part = 0; part < 2; ++part) {
    // part 0: L_ik with (L row i, Ut row k, Ut.inv_kk); part 1: Ut_ik with (Ut row i, L row k, L.inv_kk)
    const BandDesc& dr = part == 0 ? dl : du;
    const BandDesc& dc = part == 0 ? du : dl;
    T acc[4][4];
    tile_zero(acc);
    for (int j = max(0, i - dl.w); j < k; ++j)
      tile_gemm<T, false, true>(acc, pool + band_block(dr, i, j), NB, pool + band_block(dc, k, j), NB, NB, smA, smB);
    T* Aik = pool + band_block(dr, i, k);
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int p = 0; p < 4; ++p) Aik[(ty * 4 + q) * NB + tx * 4 + p] -= acc[q][p];
    __syncthreads();
    tile_zero(acc);
    tile_gemm<T, false, true>(acc, Aik, NB, pool + dc.oLinv + (long long)k * NB * NB, NB, NB, smA, smB);
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int p = 0; p < 4; ++p) Aik[(ty * 4 + q) * NB + tx * 4 + p] = acc[q][p];
    __syncthreads();
  }
}

template <typename T>
__global__ void __launch_bounds__(NT) k_lu_diag(const BandDesc* __restrict__ bl, const BandDesc* __restrict__ bu,
                                                T* __restrict__ pool, int k, int* __restrict__ err) {
  const BandDesc dl = bl[blockIdx.x], du = bu[blockIdx.x];
  if (k >= dl.nb) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* a = reinterpret_cast<T*>(smraw);
  T* inv = a + NB * (NB + 1);
  T* smA = inv + NB * (NB + 1);
  lu_diag_step<T>(dl, du, pool, k, err, a, inv, smA, smA + SM_TILE);
}

template <typename T>
__global__ void __launch_bounds__(NT) k_lu_off(const BandDesc* __restrict__ bl, const BandDesc* __restrict__ bu,
                                               T* __restrict__ pool, int k) {
  const BandDesc dl = bl[blockIdx.y], du = bu[blockIdx.y];
  const int i = k + 1 + blockIdx.x;
  if (k >= dl.nb || i >= dl.nb || i - k > dl.w) return;
  __shared__ __align__(16) T smA[SM_TILE];
  __shared__ __align__(16) T smB[SM_TILE];
  lu_off_step<T>(dl, du, pool, k, i, smA, smB);
}

// entry (r, c) of a general matrix into the L / Ut bands (diagonal blocks whole in L)
template <typename T>
__device__ __forceinline__ T& lu_slot(const BandDesc& dl, const BandDesc& du, T* pool, int r, int c) {
  return (c / NB <= r / NB) ? pool[band_block(dl, r / NB, c / NB) + (r % NB) * NB + c % NB]
                            : pool[band_block(du, c / NB, r / NB) + (c % NB) * NB + r % NB];
}

// one step for every system (one CTA per system)
template <typename T>
__global__ void __launch_bounds__(NT) k_chol_diag(const BandDesc* __restrict__ bd, T* __restrict__ pool, int k,
                                                  int* __restrict__ err) {
  const BandDesc d = bd[blockIdx.x];
  if (k >= d.nb) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* a = reinterpret_cast<T*>(smraw);
  T* inv = a + NB * (NB + 1);
  T* smA = inv + NB * (NB + 1);
  chol_diag_step<T>(d, pool, k, err, a, inv, smA, smA + SM_TILE);
}

// Right-looking steps (the trailing blocks already hold A minus the updates of
// the earlier steps): the diagonal factor, then the panel L_ik = A_ik Linv_kk^T,
// then the trailing update A_ij -= L_ik L_jk^T of every block pair k < j <= i,
// one CTA per block (pair).  For one dense system (the coarse problem) this
// spreads each step over many CTAs, where the left-looking steps leave a few
// CTAs with long chains of block products.
template <typename T>
__global__ void __launch_bounds__(NT) k_chol_rl_diag(const BandDesc* __restrict__ bd, T* __restrict__ pool, int k,
                                                     int* __restrict__ err) {
  const BandDesc d = bd[blockIdx.x];
  if (k >= d.nb) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* a = reinterpret_cast<T*>(smraw);
  T* inv = a + NB * (NB + 1);
  T* smA = inv + NB * (NB + 1);
  chol_diag_step<T>(d, pool, k, err, a, inv, smA, smA + SM_TILE, false);
}

template <typename T>
__global__ void __launch_bounds__(NT) k_chol_rl_panel(const BandDesc* __restrict__ bd, T* __restrict__ pool, int k) {
  const BandDesc d = bd[blockIdx.y];
  const int i = k + 1 + blockIdx.x;
  if (k >= d.nb || i >= d.nb || i - k > d.w) return;
  __shared__ __align__(16) T smA[SM_TILE];
  __shared__ __align__(16) T smB[SM_TILE];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
  tile_zero(acc);
  T* Aik = pool + band_block(d, i, k);
  tile_gemm<T, false, true>(acc, Aik, NB, pool + d.oLinv + (long long)k * NB * NB, NB, NB, smA, smB);
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int p = 0; p < 4; ++p) Aik[(ty * 4 + q) * NB + tx * 4 + p] = acc[q][p];
}

template <typename T>
__global__ void __launch_bounds__(NT) k_chol_rl_update(const BandDesc* __restrict__ bd, T* __restrict__ pool, int k) {
  const BandDesc d = bd[blockIdx.y];
  if (k >= d.nb) return;
  // block pair (i, j), k < j <= i, from the position in the lower triangle
  const int p = blockIdx.x;
  int ii = (int)((sqrt(8.0 * p + 1.0) - 1.0) * 0.5);
  while ((ii + 1) * (ii + 2) / 2 <= p) ++ii;
  while (ii * (ii + 1) / 2 > p) --ii;
  const int jj = p - ii * (ii + 1) / 2;
  const int i = k + 1 + ii, j = k + 1 + jj;
  if (i >= d.nb || i - k > d.w || j - k > d.w) return;
  __shared__ __align__(16) T smA[SM_TILE];
  __shared__ __align__(16) T smB[SM_TILE];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
  tile_zero(acc);
  tile_gemm<T, false, true>(acc, pool + band_block(d, i, k), NB, pool + band_block(d, j, k), NB, NB, smA, smB);
  T* Aij = pool + band_block(d, i, j);
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int p2 = 0; p2 < 4; ++p2) Aij[(ty * 4 + q) * NB + tx * 4 + p2] -= acc[q][p2];
}

template <typename T>
__global__ void __launch_bounds__(NT) k_chol_off(const BandDesc* __restrict__ bd, T* __restrict__ pool, int k) {
  const BandDesc d = bd[blockIdx.y];
  const int i = k + 1 + blockIdx.x;
  if (k >= d.nb || i >= d.nb || i - k > d.w) return;
  __shared__ __align__(16) T smA[SM_TILE];
  __shared__ __align__(16) T smB[SM_TILE];
  chol_off_step<T>(d, pool, k, i, smA, smB);
}

// forward step k: B_k = Linv_kk (B_k - sum_j L_kj B_j), one 64-column tile per CTA
template <typename T>
__global__ void __launch_bounds__(NT) k_trsm_fwd(const BandDesc* __restrict__ bd, const T* __restrict__ Lpool,
                                                 T* __restrict__ Bpool, int k) {
  const BandDesc d = bd[blockIdx.y];
  const int c0 = blockIdx.x * NB;
  if (k >= d.nb || c0 >= d.ncol) return;
  __shared__ __align__(16) T smA[SM_TILE];
  __shared__ __align__(16) T smB[SM_TILE];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int ld = d.ncol;
  T* B = Bpool + d.oB;
  T acc[4][4];
  tile_zero(acc);
  for (int j = max(0, k - d.w); j < k; ++j)
    tile_gemm<T, false, false>(acc, Lpool + band_block(d, k, j), NB, B + (long long)j * NB * ld + c0, ld, NB, smA, smB);
  T* Bk = B + (long long)k * NB * ld + c0;
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int p = 0; p < 4; ++p) Bk[(long long)(ty * 4 + q) * ld + tx * 4 + p] -= acc[q][p];
  __syncthreads();
  tile_zero(acc);
  tile_gemm<T, false, false>(acc, Lpool + d.oLinv + (long long)k * NB * NB, NB, Bk, ld, NB, smA, smB);
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int p = 0; p < 4; ++p) Bk[(long long)(ty * 4 + q) * ld + tx * 4 + p] = acc[q][p];
}

// backward step k: B_k = Linv_kk^T (B_k - sum_{i>k} L_ik^T B_i)
template <typename T>
__global__ void __launch_bounds__(NT) k_trsm_bwd(const BandDesc* __restrict__ bd, const T* __restrict__ Lpool,
                                                 T* __restrict__ Bpool, int k) {
  const BandDesc d = bd[blockIdx.y];
  const int c0 = blockIdx.x * NB;
  if (k >= d.nb || c0 >= d.ncol) return;
  __shared__ __align__(16) T smA[SM_TILE];
  __shared__ __align__(16) T smB[SM_TILE];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int ld = d.ncol;
  T* B = Bpool + d.oB;
  T acc[4][4];
  tile_zero(acc);
  int iend = min(d.nb - 1, k + d.w);
  for (int i = k + 1; i <= iend; ++i)
    tile_gemm<T, true, false>(acc, Lpool + band_block(d, i, k), NB, B + (long long)i * NB * ld + c0, ld, NB, smA, smB);
  T* Bk = B + (long long)k * NB * ld + c0;
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int p = 0; p < 4; ++p) Bk[(long long)(ty * 4 + q) * ld + tx * 4 + p] -= acc[q][p];
  __syncthreads();
  tile_zero(acc);
  tile_gemm<T, true, false>(acc, Lpool + d.oLinv + (long long)k * NB * NB, NB, Bk, ld, NB, smA, smB);
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int p = 0; p < 4; ++p) Bk[(long long)(ty * 4 + q) * ld + tx * 4 + p] = acc[q][p];
}

// --------------------------------------------------- matrix construction
struct CsrView {
  const int* ptr;     // global row pointers (absolute indices into col/val)
  const int* col;
  const double* val;
};

// interior block into block-band storage; padding rows get a unit diagonal
template <typename T>
__global__ void k_fill_band(const DevSub* __restrict__ ds, CsrView koo, T* __restrict__ pool,
                            const BandDesc* __restrict__ bd) {
  const DevSub s = ds[blockIdx.y];
  const BandDesc d = bd[blockIdx.y];
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= s.NO) return;
  if (r >= s.no) {
    pool[band_block(d, r / NB, r / NB) + (r % NB) * NB + r % NB] = T(1);
    return;
  }
  const int* ptr = koo.ptr + s.koo;
  for (int q = ptr[r]; q < ptr[r + 1]; ++q) {
    int c = koo.col[q];
    if (c <= r) pool[band_block(d, r / NB, c / NB) + (r % NB) * NB + c % NB] = T(koo.val[q]);
  }
}

// general interior block into the L / Ut bands; padding rows get a unit diagonal
template <typename T>
__global__ void k_fill_band_lu(const DevSub* __restrict__ ds, CsrView koo, T* __restrict__ pool,
                               const BandDesc* __restrict__ bl, const BandDesc* __restrict__ bu) {
  const DevSub s = ds[blockIdx.y];
  const BandDesc dl = bl[blockIdx.y], du = bu[blockIdx.y];
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= s.NO) return;
  if (r >= s.no) {
    pool[band_block(dl, r / NB, r / NB) + (r % NB) * NB + r % NB] = T(1);
    return;
  }
  const int* ptr = koo.ptr + s.koo;
  for (int q = ptr[r]; q < ptr[r + 1]; ++q) lu_slot<T>(dl, du, pool, r, koo.col[q]) = T(koo.val[q]);
}

// RHS of the interior solves: [A_oi | f_o | 0], NO x NR
template <typename T>
__global__ void k_fill_rhs(const DevSub* __restrict__ ds, CsrView koi, const double* __restrict__ fo,
                           const long long* __restrict__ fo_off, T* __restrict__ pool) {
  const DevSub s = ds[blockIdx.y];
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= s.no) return;
  T* B = pool + s.oXc + (long long)r * s.NR;
  const int* ptr = koi.ptr + s.koi;
  for (int q = ptr[r]; q < ptr[r + 1]; ++q) B[koi.col[q]] = T(koi.val[q]);
  B[s.ni] = T(fo[fo_off[blockIdx.y] + r]);
}

// Refinement residual of the interior solves, FP64-accurate on FP32 pipes:
// R = [A_oi | f_o] - A_oo X, written as FP32 into component `outcomp` (and
// into component `copycomp` too when that is >= 0).  X is component 0 (an
// exact FP32 value, xpair = 0) or the FP32 pair held in components 0 and 1
// (xpair = 1).  One CTA per RES_ROWS interior rows; each
// thread owns groups of 4 adjacent columns (float4 loads of X), the rows'
// matrix entries are staged in shared memory with their X row offsets, and
// the CTA walks its rows in order so that the band neighbours they share are
// served from L1.  Padding columns and rows are written as zero.
constexpr int RES_ROWS = 8;
constexpr int RES_MAXNZ = 96;
__global__ void __launch_bounds__(128) k_residual_df(const DevSub* __restrict__ ds, CsrView koo, CsrView koi,
                                                     const double* __restrict__ fo,
                                                     const long long* __restrict__ fo_off, float* __restrict__ pool,
                                                     int xpair, int outcomp, int copycomp = -1,
                                                     const int* __restrict__ active = nullptr) {
  if (active && !active[blockIdx.y]) return;  // a system whose refinement has converged
  const DevSub s = ds[blockIdx.y];
  const int r0 = blockIdx.x * RES_ROWS;
  if (r0 >= s.NO) return;
  __shared__ int soff[RES_ROWS][RES_MAXNZ];       // X row offsets (row * NR) of the A_oo entries
  __shared__ dfloat sval[RES_ROWS][RES_MAXNZ];    // -A_oo entries
  __shared__ int bcol[RES_ROWS][RES_MAXNZ];       // columns of [A_oi | f_o]
  __shared__ dfloat bval[RES_ROWS][RES_MAXNZ];
  __shared__ int nnz[RES_ROWS], nb[RES_ROWS];
  const int nrow = min(RES_ROWS, s.NO - r0);
  const int tid = threadIdx.x;
  if (tid < RES_ROWS) {
    const int r = r0 + tid;
    if (tid < nrow && r < s.no) {
      const int* p = koo.ptr + s.koo;
      const int* pb = koi.ptr + s.koi;
      nnz[tid] = min(RES_MAXNZ, p[r + 1] - p[r]);
      nb[tid] = min(RES_MAXNZ - 1, pb[r + 1] - pb[r]) + 1;
    } else {
      nnz[tid] = 0;
      nb[tid] = 0;
    }
  }
  __syncthreads();
  for (int rr = 0; rr < nrow; ++rr) {
    const int r = r0 + rr;
    if (r >= s.no) break;
    const int* p = koo.ptr + s.koo;
    for (int q = tid; q < nnz[rr]; q += blockDim.x) {
      soff[rr][q] = koo.col[p[r] + q] * s.NR;
      sval[rr][q] = df_from_double(-koo.val[p[r] + q]);
    }
    const int* pb = koi.ptr + s.koi;
    for (int q = tid; q < nb[rr] - 1; q += blockDim.x) {
      bcol[rr][q] = koi.col[pb[r] + q];
      bval[rr][q] = df_from_double(koi.val[pb[r] + q]);
    }
    if (tid == 0) {
      bcol[rr][nb[rr] - 1] = s.ni;
      bval[rr][nb[rr] - 1] = df_from_double(fo[fo_off[blockIdx.y] + r]);
    }
  }
  __syncthreads();
  const long long comp = (long long)s.NO * s.NR;
  const float* X0 = pool + s.oXc;
  const float* X1 = X0 + comp;
  float* out = pool + s.oXc + (long long)outcomp * comp;
  float* out2 = copycomp >= 0 ? pool + s.oXc + (long long)copycomp * comp : nullptr;
  const int ngrp = s.NR / 4;
  for (int gidx = tid; gidx < ngrp; gidx += blockDim.x) {
    const int c = 4 * gidx;
    for (int rr = 0; rr < nrow; ++rr) {
      const int r = r0 + rr;
      float4 res = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r < s.no && c <= s.ni) {
        dfacc a0, a1, a2, a3;
        for (int q = 0; q < nb[rr]; ++q) {
          const int d = bcol[rr][q] - c;
          if ((unsigned)d < 4u) {
            const dfloat v = bval[rr][q];
            if (d == 0) a0.add_df(v);
            else if (d == 1) a1.add_df(v);
            else if (d == 2) a2.add_df(v);
            else a3.add_df(v);
          }
        }
        const int n = nnz[rr];
        if (xpair) {
          for (int q = 0; q < n; ++q) {
            const dfloat a = sval[rr][q];
            const int o = soff[rr][q] + c;
            const float4 h = *reinterpret_cast<const float4*>(X0 + o);
            const float4 l = *reinterpret_cast<const float4*>(X1 + o);
            a0.fma_df(a, dfloat{h.x, l.x});
            a1.fma_df(a, dfloat{h.y, l.y});
            a2.fma_df(a, dfloat{h.z, l.z});
            a3.fma_df(a, dfloat{h.w, l.w});
          }
        } else {
          for (int q = 0; q < n; ++q) {
            const dfloat a = sval[rr][q];
            const float4 h = *reinterpret_cast<const float4*>(X0 + soff[rr][q] + c);
            a0.fma_df(a, h.x);
            a1.fma_df(a, h.y);
            a2.fma_df(a, h.z);
            a3.fma_df(a, h.w);
          }
        }
        res = make_float4(a0.value().hi, a1.value().hi, a2.value().hi, a3.value().hi);
        // columns beyond the rhs column are padding
        if (c + 1 > s.ni) res.y = 0.f;
        if (c + 2 > s.ni) res.z = 0.f;
        if (c + 3 > s.ni) res.w = 0.f;
      }
      *reinterpret_cast<float4*>(out + (long long)r * s.NR + c) = res;
      if (out2) *reinterpret_cast<float4*>(out2 + (long long)r * s.NR + c) = res;
    }
  }
}

// largest |component| per subdomain (refinement diagnostics; FP32 bit patterns
// of non-negative values order like integers)
__global__ void k_comp_maxabs(const DevSub* __restrict__ ds, const float* __restrict__ pool, int comp_id,
                              int* __restrict__ out) {
  const DevSub s = ds[blockIdx.y];
  const long long comp = (long long)s.NO * s.NR;
  const float* X = pool + s.oXc + (long long)comp_id * comp;
  float m = 0.f;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < comp; e += (long long)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(X[e]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out + blockIdx.y, __float_as_int(m));
}

// Schur complement S = A_ii - A_io (X_0 + X_1), FP64-accurate, plus the
// subdomain part of the reduced rhs g = f_i - A_io X(:, ni), where X_0 + X_1
// is the refined interior solution held as an (unnormalised) FP32 pair.
// Mixed precision stores S as FP32 (hi, lo) pairs.
__global__ void __launch_bounds__(128) k_schur_df(const DevSub* __restrict__ ds, CsrView kio, CsrView kii,
                                                  const float* __restrict__ pool, float2* __restrict__ Spool,
                                                  const double* __restrict__ fi, double* __restrict__ grep) {
  const DevSub s = ds[blockIdx.y];
  const int i = blockIdx.x;
  if (i >= s.NI) return;
  float2* Srow = Spool + s.oS + (long long)i * s.NI;
  if (i >= s.ni) {
    for (int c = threadIdx.x; c < s.NI; c += blockDim.x) Srow[c] = make_float2(0.f, 0.f);
    return;
  }
  __shared__ int scol[128];
  __shared__ dfloat sval[128];
  __shared__ int dcol[128];
  __shared__ dfloat dval[128];
  __shared__ int nnz, nd;
  if (threadIdx.x == 0) {
    const int* p = kio.ptr + s.kio;
    nnz = min(128, p[i + 1] - p[i]);
    const int* pd = kii.ptr + s.kii;
    nd = min(128, pd[i + 1] - pd[i]);
  }
  __syncthreads();
  {
    const int* p = kio.ptr + s.kio;
    for (int q = threadIdx.x; q < nnz; q += blockDim.x) {
      scol[q] = kio.col[p[i] + q];
      sval[q] = df_from_double(-kio.val[p[i] + q]);
    }
    const int* pd = kii.ptr + s.kii;
    for (int q = threadIdx.x; q < nd; q += blockDim.x) {
      dcol[q] = kii.col[pd[i] + q];
      dval[q] = df_from_double(kii.val[pd[i] + q]);
    }
  }
  __syncthreads();
  const long long comp = (long long)s.NO * s.NR;
  const float* X0 = pool + s.oXc;
  const float* X1 = X0 + comp;
  for (int c = threadIdx.x; c <= s.ni; c += blockDim.x) {
    dfacc acc;
    if (c < s.ni) {
      for (int q = 0; q < nd; ++q)
        if (dcol[q] == c) acc.add_df(dval[q]);
    } else {
      acc.add_df(df_from_double(fi[s.rep + i]));
    }
    for (int q = 0; q < nnz; ++q) {
      long long o = (long long)scol[q] * s.NR + c;
      acc.fma_df(sval[q], dfloat{X0[o], X1[o]});
    }
    if (c < s.ni) {
      dfloat v = acc.value();
      Srow[c] = make_float2(v.hi, v.lo);
    } else {
      grep[s.rep + i] = acc.to_double();
    }
  }
  for (int c = s.ni + threadIdx.x; c < s.NI; c += blockDim.x) Srow[c] = make_float2(0.f, 0.f);
}

// plain FP64 counterpart of k_schur_df (single solution component)
__global__ void __launch_bounds__(128) k_schur_f64(const DevSub* __restrict__ ds, CsrView kio, CsrView kii,
                                                   const double* __restrict__ pool, double* __restrict__ Spool,
                                                   const double* __restrict__ fi, double* __restrict__ grep) {
  const DevSub s = ds[blockIdx.y];
  const int i = blockIdx.x;
  if (i >= s.NI) return;
  double* Srow = Spool + s.oS + (long long)i * s.NI;
  if (i >= s.ni) {
    for (int c = threadIdx.x; c < s.NI; c += blockDim.x) Srow[c] = 0.0;
    return;
  }
  const int* p = kio.ptr + s.kio;
  const int* pd = kii.ptr + s.kii;
  for (int c = threadIdx.x; c <= s.ni; c += blockDim.x) {
    double acc = 0.0;
    if (c < s.ni) {
      for (int q = pd[i]; q < pd[i + 1]; ++q)
        if (kii.col[q] == c) acc += kii.val[q];
    } else {
      acc = fi[s.rep + i];
    }
    for (int q = p[i]; q < p[i + 1]; ++q) acc -= kio.val[q] * pool[s.oXc + (long long)kio.col[q] * s.NR + c];
    if (c < s.ni) Srow[c] = acc;
    else grep[s.rep + i] = acc;
  }
  for (int c = s.ni + threadIdx.x; c < s.NI; c += blockDim.x) Srow[c] = 0.0;
}

// M = (M + M^T) / 2 on the leading n x n block of a row-major NI x NI
// matrix (the computed Schur complement and preconditioner block are
// symmetric only up to rounding).  Tile pairs (I, J) and (J, I) go through
// shared memory so both reads and writes are coalesced.
template <typename E>
__device__ __forceinline__ E sym_avg(E a, E b) { return E(0.5) * (a + b); }
template <>
__device__ __forceinline__ float2 sym_avg<float2>(float2 a, float2 b) {
  dfacc acc;
  acc.add(a.x); acc.add(b.x); acc.c += a.y + b.y;
  dfloat v = acc.value();
  return make_float2(0.5f * v.hi, 0.5f * v.lo);
}

template <typename E>
__global__ void k_symmetrize(const DevSub* __restrict__ ds, E* __restrict__ pool, int which) {
  const DevSub s = ds[blockIdx.z];
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bj < bi || bi * 32 >= s.NI || bj * 32 >= s.NI) return;
  E* M = pool + (which == 0 ? s.oS : s.oZ);
  __shared__ E ta[32][33], tb[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    ta[r][tx] = M[(long long)(bi * 32 + r) * s.NI + bj * 32 + tx];
    tb[r][tx] = M[(long long)(bj * 32 + r) * s.NI + bi * 32 + tx];
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    int gi = bi * 32 + r, gj = bj * 32 + tx;
    if (gi < s.ni && gj < s.ni) M[(long long)gi * s.NI + gj] = sym_avg(ta[r][tx], tb[tx][r]);
    int hi = bj * 32 + r, hj = bi * 32 + tx;
    if (bi != bj && hi < s.ni && hj < s.ni) M[(long long)hi * s.NI + hj] = sym_avg(tb[r][tx], ta[tx][r]);
  }
}

template <typename T, typename ST>
__device__ __forceinline__ T schur_entry(const ST* S, long long idx);
template <>
__device__ __forceinline__ float schur_entry<float, float2>(const float2* S, long long idx) { return S[idx].x; }
template <>
__device__ __forceinline__ double schur_entry<double, double>(const double* S, long long idx) { return S[idx]; }

// Preconditioner block Srho = S + rho * C~^T C~ (rows of C scaled to unit norm),
// lower blocks in dense-block storage; unit diagonal on the padding.  On the
// constraint set C z = 0 it equals S, so the constrained solve is unchanged.
template <typename T, typename ST>
__global__ void k_fill_srho(const DevSub* __restrict__ ds, const ST* __restrict__ Spool, T* __restrict__ pool,
                            const BandDesc* __restrict__ bd) {
  const DevSub s = ds[blockIdx.z];
  const BandDesc d = bd[blockIdx.z];
  int i = blockIdx.y * 16 + threadIdx.y, j = blockIdx.x * 16 + threadIdx.x;
  if (i >= s.NI || j > i) return;
  T v;
  if (i < s.ni && j < s.ni) v = schur_entry<T, ST>(Spool + s.oS, (long long)i * s.NI + j);
  else v = (i == j) ? T(1) : T(0);
  pool[band_block(d, i / NB, j / NB) + (i % NB) * NB + j % NB] = v;
}

template <typename T>
__global__ void k_add_penalty(const DevSub* __restrict__ ds, const int* __restrict__ cptr, const int* __restrict__ ccol,
                              const double* __restrict__ cval, T* __restrict__ pool, const BandDesc* __restrict__ bd) {
  const DevSub s = ds[blockIdx.y];
  const BandDesc d = bd[blockIdx.y];
  const int* p = cptr + s.cptr;
  // rows one after the other: rows of one coarse node (several constraints on
  // a face) share their entries, and a fixed order keeps the sum deterministic
  for (int r = 0; r < s.nc; ++r) {
    const int q0 = p[r], n = p[r + 1] - q0;
    double nrm = 0.0;
    for (int q = 0; q < n; ++q) nrm += cval[q0 + q] * cval[q0 + q];
    const double sc = s.rho / nrm;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      int a = e / n, b = e % n;
      int i = ccol[q0 + a], j = ccol[q0 + b];
      if (j > i) continue;
      pool[band_block(d, i / NB, j / NB) + (i % NB) * NB + j % NB] += T(sc * cval[q0 + a] * cval[q0 + b]);
    }
    __syncthreads();
  }
}

// general Srho = S + rho * C~^T C~ into the L / Ut bands (every entry; unit
// diagonal on the padding)
template <typename T, typename ST>
__global__ void k_fill_srho_lu(const DevSub* __restrict__ ds, const ST* __restrict__ Spool, T* __restrict__ pool,
                               const BandDesc* __restrict__ bl, const BandDesc* __restrict__ bu) {
  const DevSub s = ds[blockIdx.z];
  const BandDesc dl = bl[blockIdx.z], du = bu[blockIdx.z];
  int i = blockIdx.y * 16 + threadIdx.y, j = blockIdx.x * 16 + threadIdx.x;
  if (i >= s.NI || j >= s.NI) return;
  T v;
  if (i < s.ni && j < s.ni) v = schur_entry<T, ST>(Spool + s.oS, (long long)i * s.NI + j);
  else v = (i == j) ? T(1) : T(0);
  lu_slot<T>(dl, du, pool, i, j) = v;
}

template <typename T>
__global__ void k_add_penalty_lu(const DevSub* __restrict__ ds, const int* __restrict__ cptr,
                                 const int* __restrict__ ccol, const double* __restrict__ cval, T* __restrict__ pool,
                                 const BandDesc* __restrict__ bl, const BandDesc* __restrict__ bu) {
  const DevSub s = ds[blockIdx.y];
  const BandDesc dl = bl[blockIdx.y], du = bu[blockIdx.y];
  const int* p = cptr + s.cptr;
  for (int r = 0; r < s.nc; ++r) {  // rows in a fixed order (shared entries, deterministic sums)
    const int q0 = p[r], n = p[r + 1] - q0;
    double nrm = 0.0;
    for (int q = 0; q < n; ++q) nrm += cval[q0 + q] * cval[q0 + q];
    const double sc = s.rho / nrm;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      int a = e / n, b = e % n;
      lu_slot<T>(dl, du, pool, ccol[q0 + a], ccol[q0 + b]) += T(sc * cval[q0 + a] * cval[q0 + b]);
    }
    __syncthreads();
  }
}

// dual input Y_dual = Srho^-T C^T = V^T C^T from the explicit inverse V = Srho^-1
// (the adjoint solve of module_dd.f90:5687-5757 without a transposed factor solve)
template <typename T>
__global__ void k_ydual(const DevSub* __restrict__ ds, const int* __restrict__ cptr, const int* __restrict__ ccol,
                        const double* __restrict__ cval, T* __restrict__ pool) {
  const DevSub s = ds[blockIdx.y];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= s.NI * s.ncp) return;
  const int i = e / s.ncp, c = e % s.ncp;
  double t = 0.0;
  if (c < s.nc && i < s.ni) {
    const int* p = cptr + s.cptr;
    for (int k = p[c]; k < p[c + 1]; ++k) t += cval[k] * (double)pool[s.oBs + (long long)ccol[k] * s.NRC + i];
  }
  pool[s.oYd + e] = T(t);
}

// RHS [I | C^T | 0] of the preconditioner solves
template <typename T>
__global__ void k_fill_rhs_srho(const DevSub* __restrict__ ds, const int* __restrict__ cptr,
                                const int* __restrict__ ccol, const double* __restrict__ cval, T* __restrict__ pool) {
  const DevSub s = ds[blockIdx.y];
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < s.NI) pool[s.oBs + (long long)i * s.NRC + i] = T(1);
  if (i < s.nc) {
    const int* p = cptr + s.cptr;
    for (int q = p[i]; q < p[i + 1]; ++q) pool[s.oBs + (long long)ccol[q] * s.NRC + s.NI + i] = T(cval[q]);
  }
}

// G = C Y (nc x nc), its Cholesky factor and inverse, FP64 (one CTA per subdomain)
template <typename T>
__global__ void __launch_bounds__(256) k_small_g(const DevSub* __restrict__ ds, const int* __restrict__ cptr,
                                                 const int* __restrict__ ccol, const double* __restrict__ cval,
                                                 const T* __restrict__ pool, double* __restrict__ small,
                                                 int* __restrict__ err, int general) {
  const DevSub s = ds[blockIdx.x];
  const int nc = s.nc, ld = max(1, s.nc);
  extern __shared__ __align__(16) unsigned char smraw[];
  double* g = reinterpret_cast<double*>(smraw);  // nc x nc
  double* inv = g + ld * ld;
  const int* p = cptr + s.cptr;
  for (int e = threadIdx.x; e < nc * nc; e += blockDim.x) {
    int r = e / nc, q = e % nc;
    double t = 0.0;
    for (int k = p[r]; k < p[r + 1]; ++k) t += cval[k] * (double)pool[s.oBs + (long long)ccol[k] * s.NRC + s.NI + q];
    g[r * ld + q] = t;
  }
  __syncthreads();
  if (general) {
    // G = C Y of a general matrix: Gauss-Jordan inverse with partial pivoting
    __shared__ int pivrow;
    for (int e = threadIdx.x; e < nc * nc; e += blockDim.x) inv[(e / nc) * ld + e % nc] = (e / nc == e % nc) ? 1.0 : 0.0;
    __syncthreads();
    for (int c = 0; c < nc; ++c) {
      if (threadIdx.x == 0) {
        int pr = c;
        for (int r = c + 1; r < nc; ++r)
          if (fabs(g[r * ld + c]) > fabs(g[pr * ld + c])) pr = r;
        if (!(fabs(g[pr * ld + c]) > 0.0)) { atomicOr(err, DE_PIVOT); g[pr * ld + c] = 1.0; }
        pivrow = pr;
      }
      __syncthreads();
      const int pr = pivrow;
      if (pr != c)
        for (int q = threadIdx.x; q < nc; q += blockDim.x) {
          double t = g[c * ld + q]; g[c * ld + q] = g[pr * ld + q]; g[pr * ld + q] = t;
          t = inv[c * ld + q]; inv[c * ld + q] = inv[pr * ld + q]; inv[pr * ld + q] = t;
        }
      __syncthreads();
      const double dinv = 1.0 / g[c * ld + c];
      __syncthreads();
      for (int q = threadIdx.x; q < nc; q += blockDim.x) { g[c * ld + q] *= dinv; inv[c * ld + q] *= dinv; }
      __syncthreads();
      for (int e = threadIdx.x; e < nc * nc; e += blockDim.x) {
        const int r = e / nc, q = e % nc;
        if (r == c) continue;
        const double f = g[r * ld + c];
        if (q != c) g[r * ld + q] -= f * g[c * ld + q];
        inv[r * ld + q] -= f * inv[c * ld + q];
      }
      __syncthreads();
      for (int r = threadIdx.x; r < nc; r += blockDim.x) if (r != c) g[r * ld + c] = 0.0;
      __syncthreads();
    }
    double* Gi = small + s.oGinv;
    double* Ac = small + s.oAc;
    for (int e = threadIdx.x; e < s.ncp * s.ncp; e += blockDim.x) {
      int r = e / s.ncp, q = e % s.ncp;
      double t = (r < nc && q < nc) ? inv[r * ld + q] : 0.0;
      Gi[e] = t;
      if (r < nc && r == q) {  // Phi_dual^T S Phi = G^-1 - rho D^2 as for symmetric matrices
        double nrm = 0.0;
        for (int k = p[r]; k < p[r + 1]; ++k) nrm += cval[k] * cval[k];
        t -= s.rho / nrm;
      }
      Ac[e] = t;
    }
    return;
  }
  for (int e = threadIdx.x; e < nc * nc; e += blockDim.x) {
    int r = e / nc, q = e % nc;
    if (q > r) {
      double m = 0.5 * (g[r * ld + q] + g[q * ld + r]);
      g[r * ld + q] = m;
      g[q * ld + r] = m;
    }
  }
  __syncthreads();
  for (int c = 0; c < nc; ++c) {
    if (threadIdx.x == 0) {
      double v = g[c * ld + c];
      if (!(v > 0.0)) { atomicOr(err, DE_PIVOT); v = 1.0; }
      g[c * ld + c] = sqrt(v);
    }
    __syncthreads();
    for (int r = c + 1 + threadIdx.x; r < nc; r += blockDim.x) g[r * ld + c] /= g[c * ld + c];
    __syncthreads();
    int m = nc - c - 1;
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
      int r = c + 1 + e / m, q = c + 1 + e % m;
      if (q <= r) g[r * ld + q] -= g[r * ld + c] * g[q * ld + c];
    }
    __syncthreads();
  }
  // L^-1 column by column, then Ginv = L^-T L^-1
  if (threadIdx.x < nc) {
    int j = threadIdx.x;
    for (int i = 0; i < j; ++i) inv[i * ld + j] = 0.0;
    inv[j * ld + j] = 1.0 / g[j * ld + j];
    for (int i = j + 1; i < nc; ++i) {
      double t = 0.0;
      for (int m = j; m < i; ++m) t += g[i * ld + m] * inv[m * ld + j];
      inv[i * ld + j] = -t / g[i * ld + i];
    }
  }
  __syncthreads();
  // G^-1 and the local coarse matrix.  With Srho = S + C^T (rho D^2) C
  // (D = diag(1/|c_r|)), Y = Srho^-1 C^T and Phi = Y G^-1:  Srho Phi = C^T G^-1
  // and C Phi = I, hence Phi^T S Phi = G^-1 - rho D^2 (= -lambda of the
  // reference's augmented solve, module_dd.f90:5615-5625).
  double* Gi = small + s.oGinv;
  double* Ac = small + s.oAc;
  for (int e = threadIdx.x; e < s.ncp * s.ncp; e += blockDim.x) {
    int r = e / s.ncp, q = e % s.ncp;
    double t = 0.0;
    if (r < nc && q < nc)
      for (int m = max(r, q); m < nc; ++m) t += inv[m * ld + r] * inv[m * ld + q];
    Gi[e] = t;
    if (r < nc && r == q) {
      double nrm = 0.0;
      for (int k = p[r]; k < p[r + 1]; ++k) nrm += cval[k] * cval[k];
      t -= s.rho / nrm;
    }
    Ac[e] = t;
  }
}

// Phi = Y Ginv  (NI x ncp, preconditioner precision)
template <typename T>
__global__ void k_phi(const DevSub* __restrict__ ds, const T* __restrict__ pool, const double* __restrict__ small,
                      T* __restrict__ pcpool, int dual) {
  const DevSub s = ds[blockIdx.y];
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= s.NI * s.ncp) return;
  int i = e / s.ncp, c = e % s.ncp;
  double t = 0.0;
  if (c < s.nc && i < s.ni) {
    const double* gi = small + s.oGinv;
    if (dual) {  // Phi_dual = Y_dual G^-T
      const T* y = pool + s.oYd + (long long)i * s.ncp;
      for (int q = 0; q < s.nc; ++q) t += (double)y[q] * gi[c * s.ncp + q];
    } else {     // Phi = Y G^-1
      const T* y = pool + s.oBs + (long long)i * s.NRC + s.NI;
      for (int q = 0; q < s.nc; ++q) t += (double)y[q] * gi[q * s.ncp + c];
    }
  }
  pcpool[(dual ? s.oPhid : s.oPhi) + e] = T(t);
}

// Z = Srho^-1 - Phi Y^T on the interface block (dense, preconditioner
// precision); 16 x 16 output tiles with the Phi and Y rows staged in shared
// memory
constexpr int NCMAX = 120;
template <typename T>
__global__ void k_z(const DevSub* __restrict__ ds, const T* __restrict__ pool, T* __restrict__ pcpool, int general) {
  const DevSub s = ds[blockIdx.z];
  const int i0 = blockIdx.y * 16, j0 = blockIdx.x * 16;
  if (i0 >= s.NI || j0 >= s.NI) return;
  __shared__ T ph[16][NCMAX + 1], yy[16][NCMAX + 1];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 16 + tx;
  // Z = V - Phi Y^T, with Y_dual in place of Y for a general matrix (Z = V - Y G^-1 Y_dual^T)
  for (int e = tid; e < 16 * s.nc; e += 256) {
    int r = e / s.nc, c = e % s.nc;
    ph[r][c] = pcpool[s.oPhi + (long long)(i0 + r) * s.ncp + c];
    yy[r][c] = general ? pool[s.oYd + (long long)(j0 + r) * s.ncp + c]
                       : pool[s.oBs + (long long)(j0 + r) * s.NRC + s.NI + c];
  }
  __syncthreads();
  const int i = i0 + ty, j = j0 + tx;
  T v = T(0);
  if (i < s.ni && j < s.ni) {
    v = pool[s.oBs + (long long)i * s.NRC + j];
    for (int c = 0; c < s.nc; ++c) v -= ph[ty][c] * yy[tx][c];
  }
  pcpool[s.oZ + (long long)i * s.NI + j] = v;
}

// Symmetric matrices: Z = V - Phi Y^T and its symmetrisation (Z + Z^T) / 2 in
// one pass.  One CTA per pair of 32 x 32 tiles (bi, bj), bj >= bi, forms both
// T1 = Z[bi, bj] and T2 = Z[bj, bi] from V, Phi and Y staged in shared memory
// and writes the average of T1 and T2^T to both places: the same values as
// k_z followed by k_symmetrize, without the second pass over Z.  Only the
// lower triangle of V = Srho^-1 is read (the sweeps form only that, up to the
// 64-row diagonal blocks): V[bi, bj] = V[bj, bi]^T off the diagonal.  grid (NI/32,
// NI/32, nsub), 32 x 8 threads, dynamic shared memory 4 * 32 * (ncpmax + 1)
// elements of T (Phi and Y rows of both tiles).
template <typename T>
__global__ void __launch_bounds__(256) k_z_sym(const DevSub* __restrict__ ds, const T* __restrict__ pool,
                                               T* __restrict__ pcpool, int ncpmax) {
  const DevSub s = ds[blockIdx.z];
  const int bi = blockIdx.y, bj = blockIdx.x;
  if (bj < bi || bi * 32 >= s.NI || bj * 32 >= s.NI) return;  // padding tiles are written as zeros
  extern __shared__ __align__(16) unsigned char zs_raw[];
  const int ldc = ncpmax + 1;
  T* phi_i = reinterpret_cast<T*>(zs_raw);
  T* phi_j = phi_i + 32 * ldc;
  T* y_i = phi_j + 32 * ldc;
  T* y_j = y_i + 32 * ldc;
  __shared__ T ta[32][33], tb[32][33];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * 32 + tx;
  const int i0 = bi * 32, j0 = bj * 32, nc = s.nc;
  for (int e = tid; e < 32 * nc; e += 256) {
    const int r = e / nc, c = e % nc;
    phi_i[r * ldc + c] = pcpool[s.oPhi + (long long)(i0 + r) * s.ncp + c];
    phi_j[r * ldc + c] = pcpool[s.oPhi + (long long)(j0 + r) * s.ncp + c];
    y_i[r * ldc + c] = pool[s.oBs + (long long)(i0 + r) * s.NRC + s.NI + c];
    y_j[r * ldc + c] = pool[s.oBs + (long long)(j0 + r) * s.NRC + s.NI + c];
  }
  for (int r = ty; r < 32; r += 8) tb[r][tx] = pool[s.oBs + (long long)(j0 + r) * s.NRC + i0 + tx];
  __syncthreads();
  for (int r = ty; r < 32; r += 8) ta[r][tx] = bi == bj ? tb[r][tx] : tb[tx][r];
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    T v1 = ta[r][tx], v2 = tb[r][tx];
    for (int c = 0; c < nc; ++c) {
      v1 -= phi_i[r * ldc + c] * y_j[tx * ldc + c];
      v2 -= phi_j[r * ldc + c] * y_i[tx * ldc + c];
    }
    ta[r][tx] = v1;
    tb[r][tx] = v2;
  }
  __syncthreads();
  T* Z = pcpool + s.oZ;
  for (int r = ty; r < 32; r += 8) {
    const int gi = i0 + r, gj = j0 + tx;
    if (gi < s.NI && gj < s.NI)
      Z[(long long)gi * s.NI + gj] = (gi < s.ni && gj < s.ni) ? sym_avg(ta[r][tx], tb[tx][r]) : T(0);
    const int hi = j0 + r, hj = i0 + tx;
    if (bi != bj && hi < s.NI && hj < s.NI)
      Z[(long long)hi * s.NI + hj] = (hi < s.ni && hj < s.ni) ? sym_avg(tb[r][tx], ta[tx][r]) : T(0);
  }
}

// ---------------------------------------------------- one right-hand side
// New loads after setup (bddcml_setup_new_data_c) need v = A_oo^-1 f_o and
// g = f_i - A_io v per subdomain, with the factors already in place.

// In-place solve (L L^T) x = b of one vector per system with the block-band
// factor; grid = systems, NT threads.  x lives in shared memory during the
// sweeps; forward rows are warp dot products along the band row, backward
// columns are summed over four 16-row groups of the blocks below.
// Dynamic shared memory: (nb*NB + 5*NB) elements of T.
template <typename T>
__global__ void __launch_bounds__(NT) k_band_solve1(const BandDesc* __restrict__ bd, const T* __restrict__ pool,
                                                    T* __restrict__ xv, const long long* __restrict__ xoff,
                                                    const BandDesc* __restrict__ bdb = nullptr) {
  const BandDesc d = bd[blockIdx.x];
  const BandDesc db = bdb ? bdb[blockIdx.x] : d;  // backward factor: U^T of a general matrix, else L
  if (d.nb == 0) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  T* xs = reinterpret_cast<T*>(smraw);  // nb * NB
  T* ts = xs + d.nb * NB;                // NB
  T* part = ts + NB;                     // 4 * NB
  T* x = xv + xoff[blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n = d.nb * NB;
  for (int i = tid; i < n; i += NT) xs[i] = x[i];
  __syncthreads();
  for (int k = 0; k < d.nb; ++k) {
    const int j0 = max(0, k - d.w);
    for (int r = warp; r < NB; r += NT / 32) {  // t = x_k - sum_j L_kj x_j
      T acc = T(0);
      for (int j = j0; j < k; ++j) {
        const T* Lr = pool + band_block(d, k, j) + r * NB;
        acc += Lr[lane] * xs[j * NB + lane] + Lr[lane + 32] * xs[j * NB + lane + 32];
      }
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) ts[r] = xs[k * NB + r] - acc;
    }
    __syncthreads();
    const T* Li = pool + d.oLinv + (long long)k * NB * NB;
    for (int r = warp; r < NB; r += NT / 32) {  // x_k = Linv_kk t
      T acc = Li[r * NB + lane] * ts[lane] + Li[r * NB + lane + 32] * ts[lane + 32];
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) xs[k * NB + r] = acc;
    }
    __syncthreads();
  }
  const int c = tid & (NB - 1), grp = tid / NB;
  for (int k = d.nb - 1; k >= 0; --k) {
    T acc = T(0);  // sum_{i>k} L_ik^T x_i, rows of this thread's group
    for (int i = k + 1; i <= min(d.nb - 1, k + d.w); ++i) {
      const T* L = pool + band_block(db, i, k);
      for (int r = grp * 16; r < grp * 16 + 16; ++r) acc += L[r * NB + c] * xs[i * NB + r];
    }
    part[grp * NB + c] = acc;
    __syncthreads();
    if (tid < NB) ts[tid] = xs[k * NB + tid] - ((part[tid] + part[NB + tid]) + (part[2 * NB + tid] + part[3 * NB + tid]));
    __syncthreads();
    const T* Li = pool + db.oLinv + (long long)k * NB * NB;
    T a2 = T(0);  // x_k = Linv_kk^T t
    for (int r = grp * 16; r < grp * 16 + 16; ++r) a2 += Li[r * NB + c] * ts[r];
    part[grp * NB + c] = a2;
    __syncthreads();
    if (tid < NB) xs[k * NB + tid] = (part[tid] + part[NB + tid]) + (part[2 * NB + tid] + part[3 * NB + tid]);
    __syncthreads();
  }
  for (int i = tid; i < n; i += NT) x[i] = xs[i];
}

// x = f_o in the factor precision (padding rows zero); one vector per system
template <typename T>
__global__ void k_fill_vec1(const DevSub* __restrict__ ds, const double* __restrict__ fo,
                            const long long* __restrict__ fo_off, T* __restrict__ xv,
                            const long long* __restrict__ xoff) {
  const DevSub s = ds[blockIdx.y];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= s.NO) return;
  xv[xoff[blockIdx.y] + r] = r < s.no ? T(fo[fo_off[blockIdx.y] + r]) : T(0);
}

// r = f_o - A_oo (v0 + v1), FP64-accurate in double-float, written as FP32;
// v1 may be null (v0 is then an exact FP32 value)
__global__ void k_residual1_df(const DevSub* __restrict__ ds, CsrView koo, const double* __restrict__ fo,
                               const long long* __restrict__ fo_off, const float* __restrict__ v0,
                               const float* __restrict__ v1, float* __restrict__ rv,
                               const long long* __restrict__ xoff) {
  const DevSub s = ds[blockIdx.y];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= s.NO) return;
  const long long off = xoff[blockIdx.y];
  if (r >= s.no) { rv[off + r] = 0.f; return; }
  dfacc acc;
  acc.add_df(df_from_double(fo[fo_off[blockIdx.y] + r]));
  const int* p = koo.ptr + s.koo;
  for (int q = p[r]; q < p[r + 1]; ++q) {
    const int col = koo.col[q];
    const dfloat a = df_from_double(-koo.val[q]);
    if (v1) acc.fma_df(a, dfloat{v0[off + col], v1[off + col]});
    else acc.fma_df(a, v0[off + col]);
  }
  rv[off + r] = acc.value().hi;
}

// y += x (one vector per system)
template <typename T>
__global__ void k_add_vec1(const DevSub* __restrict__ ds, const T* __restrict__ x, T* __restrict__ y,
                           const long long* __restrict__ xoff) {
  const DevSub s = ds[blockIdx.y];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= s.NO) return;
  y[xoff[blockIdx.y] + r] += x[xoff[blockIdx.y] + r];
}

// column ni of the interior solution block X: component 0 = v0 and, for the
// double-float pair, component 1 = v1
template <typename T>
__global__ void k_put_rhs_column(const DevSub* __restrict__ ds, T* __restrict__ pool, const T* __restrict__ v0,
                                 const T* __restrict__ v1, const long long* __restrict__ xoff) {
  const DevSub s = ds[blockIdx.y];
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= s.NO) return;
  const long long off = xoff[blockIdx.y];
  T* X0 = pool + s.oXc;
  X0[(long long)r * s.NR + s.ni] = r < s.no ? v0[off + r] : T(0);
  if (v1) X0[(long long)s.NO * s.NR + (long long)r * s.NR + s.ni] = r < s.no ? v1[off + r] : T(0);
}

// g = f_i - A_io X(:, ni): the reduced-rhs column of k_schur_df / k_schur_f64
// alone, in the same operation order
__global__ void k_reduced_rhs_df(const DevSub* __restrict__ ds, CsrView kio, const float* __restrict__ pool,
                                 const double* __restrict__ fi, double* __restrict__ grep) {
  const DevSub s = ds[blockIdx.y];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.ni) return;
  const long long comp = (long long)s.NO * s.NR;
  const float* X0 = pool + s.oXc;
  const float* X1 = X0 + comp;
  dfacc acc;
  acc.add_df(df_from_double(fi[s.rep + i]));
  const int* p = kio.ptr + s.kio;
  for (int q = p[i]; q < p[i + 1]; ++q) {
    const long long o = (long long)kio.col[q] * s.NR + s.ni;
    acc.fma_df(df_from_double(-kio.val[q]), dfloat{X0[o], X1[o]});
  }
  grep[s.rep + i] = acc.to_double();
}

__global__ void k_reduced_rhs_f64(const DevSub* __restrict__ ds, CsrView kio, const double* __restrict__ pool,
                                  const double* __restrict__ fi, double* __restrict__ grep) {
  const DevSub s = ds[blockIdx.y];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.ni) return;
  double acc = fi[s.rep + i];
  const int* p = kio.ptr + s.kio;
  for (int q = p[i]; q < p[i + 1]; ++q) acc -= kio.val[q] * pool[s.oXc + (long long)kio.col[q] * s.NR + s.ni];
  grep[s.rep + i] = acc;
}

}  // namespace bddc
