// Device kernels of the BDDC solver (sm_103a).
//
// Blocked dense linear algebra on 64 x 64 tiles, batched over subdomains of
// different sizes through per-subdomain descriptors.  Each subdomain's
// interior stiffness block is a band matrix after reordering; it is stored as
// block rows of (w+1) dense 64 x 64 tiles ("block band"), so the same
// kernels serve the band factor of the interior block (small w) and the dense
// factor of the interface-sized preconditioner block (w = nb - 1).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace bddc {

constexpr int NB = 64;      // tile edge
constexpr int NT = 256;     // threads of the tile kernels (16 x 16, 4 x 4 outputs each)
constexpr int KC = 32;      // K chunk of the SIMT tile product
constexpr int KCS = NB + 4;  // row stride of a staged K chunk (spreads the transposing stores over banks)
constexpr int SM_TILE = KC * KCS;  // elements of one staged operand chunk

// error flags written by kernels (bit field), read by the host after setup
enum DevErr : int { DE_PIVOT = 1, DE_NAN = 2, DE_SMALL = 4 };

struct BandDesc {
  int nb;            // block rows (0 = nothing to do for this entry)
  int w;             // band width in blocks
  int ncol;          // RHS columns (multiple of NB)
  int pad;
  long long oL;      // offset of the block band (elements)
  long long oLinv;   // offset of the inverted diagonal blocks
  long long oB;      // offset of the RHS block (row-major, ld = ncol)
};

__host__ __device__ inline long long band_block(const BandDesc& d, int i, int j) {
  return d.oL + ((long long)i * (d.w + 1) + (j - i + d.w)) * (NB * NB);
}

// four consecutive elements from 16-byte aligned shared memory
__device__ __forceinline__ void load4(float (&v)[4], const float* p) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void load4(double (&v)[4], const double* p) {
  const double2 t0 = *reinterpret_cast<const double2*>(p);
  const double2 t1 = *reinterpret_cast<const double2*>(p + 2);
  v[0] = t0.x; v[1] = t0.y; v[2] = t1.x; v[3] = t1.y;
}

// --------------------------------------------------------------- SIMT tile
// acc(4x4 per thread) += op(A) * op(B) over K (multiple of KC), 64 x 64 output.
// A: !TA -> A[r*lda + k], TA -> A[k*lda + r];  B: !TB -> B[k*ldb + c], TB -> B[c*ldb + k]
// The next K chunk is loaded into registers while the current one is used,
// so only the first chunk's global-memory latency is exposed.
template <typename T, bool TA, bool TB>
__device__ __forceinline__ void tile_gemm(T (&acc)[4][4], const T* __restrict__ A, int lda,
                                          const T* __restrict__ B, int ldb, int K, T* smA, T* smB) {
  constexpr int PER = KC * NB / NT;  // elements of each operand per thread and chunk
  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  T ra[PER], rb[PER];
  auto fetch = [&](int k0) {
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int e = tid + i * NT;
      int r, k;
      if (!TA) { k = e % KC; r = e / KC; } else { r = e % NB; k = e / NB; }
      ra[i] = TA ? A[(long long)(k0 + k) * lda + r] : A[(long long)r * lda + k0 + k];
      int c, kk;
      if (!TB) { c = e % NB; kk = e / NB; } else { kk = e % KC; c = e / KC; }
      rb[i] = TB ? B[(long long)c * ldb + k0 + kk] : B[(long long)(k0 + kk) * ldb + c];
    }
  };
  fetch(0);
  for (int k0 = 0; k0 < K; k0 += KC) {
    // stage the chunk as smA[k][r], smB[k][c]  (KC x 64 each)
#pragma unroll
    for (int i = 0; i < PER; ++i) {
      const int e = tid + i * NT;
      int r, k;
      if (!TA) { k = e % KC; r = e / KC; } else { r = e % NB; k = e / NB; }
      smA[k * KCS + r] = ra[i];
      int c, kk;
      if (!TB) { c = e % NB; kk = e / NB; } else { kk = e % KC; c = e / KC; }
      smB[kk * KCS + c] = rb[i];
    }
    __syncthreads();
    if (k0 + KC < K) fetch(k0 + KC);
#pragma unroll
    for (int k = 0; k < KC; ++k) {
      T a[4], b[4];
      load4(a, smA + k * KCS + ty * 4);  // vector shared-memory loads
      load4(b, smB + k * KCS + tx * 4);
#pragma unroll
      for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int p = 0; p < 4; ++p) acc[q][p] += a[q] * b[p];
    }
    __syncthreads();
  }
}

template <typename T>
__device__ __forceinline__ void tile_zero(T (&acc)[4][4]) {
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int p = 0; p < 4; ++p) acc[q][p] = T(0);
}

}  // namespace bddc
