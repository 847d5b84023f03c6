// Per-iteration kernels of the BDDC-preconditioned interface PCG.
//
// Vectors live on the unique interface dofs (the reference keeps one copy per
// subdomain and makes them consistent by neighbour exchange; the values are
// the same).  Each iteration:
//   ap = sum_s R_s^T S_s R_s p           levels_sm_apply, module_levels.f90:4443-4507
//   z  = sum_s R_s^T W_s (Z_s + Phi_s Ac^-1 Phi_s^T ...) W_s R_s r
//                                        levels_pc_apply, module_levels.f90:3627-4346
//   dot products, x/r/p updates, stop test and Lanczos coefficients as in
//   krylov_bddcpcg, module_krylov.f90:545-888.
// All reductions are two-stage and run in a fixed order (deterministic).
#pragma once

#include "bddc_df.cuh"
#include "bddc_setup_kernels.cuh"

namespace bddc {

constexpr int AROWS = 32;   // matrix rows per CTA in the subdomain apply kernels
constexpr int AT = 256;     // threads of the apply kernels
constexpr int RT = 256;     // threads of the reduction kernels
constexpr int MAXPART = 1024;

struct PcgCtl {
  double rmp, pap, alpha, beta, normres2, normres0, relres, lastres, tol;
  int iter, maxit, ndecrmax, ndecr, done, reason, num_iter, nw, warn;
};

struct Owners {          // unique interface dof -> replicated positions, ascending subdomain
  const int* ptr;        // ninterface + 1
  const int* rep;        // replicated index (rep_s + i)
  const int* sub;        // subdomain of each entry
  const int* loc;        // local interface index of each entry
};

__device__ __forceinline__ double block_reduce(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  v = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;  // valid in thread 0
}

// ------------------------------------------------------- Schur operator
// y_s = S_s p_s, S_s stored as FP32 (hi, lo) pairs, double-float accumulation
__global__ void __launch_bounds__(AT) k_schur_apply_df(const DevSub* __restrict__ ds, const float2* __restrict__ Spool,
                                                       const double* __restrict__ p, const int* __restrict__ uniq,
                                                       double* __restrict__ yrep, const PcgCtl* __restrict__ ctl) {
  if (ctl && ctl->done) return;
  const DevSub s = ds[blockIdx.y];
  const int r0 = blockIdx.x * AROWS;
  if (r0 >= s.ni) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  float2* xs = reinterpret_cast<float2*>(smraw);
  for (int j = threadIdx.x; j < s.NI; j += AT) {
    double v = j < s.ni ? p[uniq[s.rep + j]] : 0.0;
    float h = (float)v;
    xs[j] = make_float2(h, (float)(v - (double)h));
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rend = min(r0 + AROWS, s.ni);
  for (int r = r0 + warp; r < rend; r += AT / 32) {
    const float4* row = reinterpret_cast<const float4*>(Spool + s.oS + (long long)r * s.NI);
    dfacc acc;
    for (int j2 = lane; j2 < s.NI / 2; j2 += 32) {
      float4 a = __ldg(row + j2);
      float2 x0 = xs[2 * j2], x1 = xs[2 * j2 + 1];
      acc.fma_df(dfloat{a.x, a.y}, dfloat{x0.x, x0.y});
      acc.fma_df(dfloat{a.z, a.w}, dfloat{x1.x, x1.y});
    }
    for (int o = 16; o > 0; o >>= 1) {
      dfacc other;
      other.s = __shfl_xor_sync(0xffffffffu, acc.s, o);
      other.c = __shfl_xor_sync(0xffffffffu, acc.c, o);
      acc.merge(other);
    }
    if (lane == 0) yrep[s.rep + r] = acc.to_double();
  }
}

// plain FP64 operator
__global__ void __launch_bounds__(AT) k_schur_apply_f64(const DevSub* __restrict__ ds, const double* __restrict__ Spool,
                                                        const double* __restrict__ p, const int* __restrict__ uniq,
                                                        double* __restrict__ yrep, const PcgCtl* __restrict__ ctl) {
  if (ctl && ctl->done) return;
  const DevSub s = ds[blockIdx.y];
  const int r0 = blockIdx.x * AROWS;
  if (r0 >= s.ni) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  double* xs = reinterpret_cast<double*>(smraw);
  for (int j = threadIdx.x; j < s.NI; j += AT) xs[j] = j < s.ni ? p[uniq[s.rep + j]] : 0.0;
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rend = min(r0 + AROWS, s.ni);
  for (int r = r0 + warp; r < rend; r += AT / 32) {
    const double2* row = reinterpret_cast<const double2*>(Spool + s.oS + (long long)r * s.NI);
    double acc = 0.0;
    for (int j2 = lane; j2 < s.NI / 2; j2 += 32) {
      double2 a = __ldg(row + j2);
      acc += a.x * xs[2 * j2] + a.y * xs[2 * j2 + 1];
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) yrep[s.rep + r] = acc;
  }
}

// ap[g] = sum of the subdomain results, zeroed at fixed dofs; partial (p, ap)
__global__ void __launch_bounds__(RT) k_assemble_dot(int n, Owners own, const double* __restrict__ yrep,
                                                     const int* __restrict__ fixed, const double* __restrict__ wsum,
                                                     const double* __restrict__ p, double* __restrict__ out,
                                                     double* __restrict__ part, const PcgCtl* __restrict__ ctl,
                                                     int zero_fixed) {
  if (ctl && ctl->done) return;
  __shared__ double sh[32];
  double loc = 0.0;
  for (int g = blockIdx.x * RT + threadIdx.x; g < n; g += gridDim.x * RT) {
    double v = 0.0;
    for (int q = own.ptr[g]; q < own.ptr[g + 1]; ++q) v += yrep[own.rep[q]];
    if (zero_fixed && fixed[g]) v = 0.0;
    out[g] = v;
    if (p) loc += wsum[g] * p[g] * v;
  }
  double t = block_reduce(loc, sh);
  if (threadIdx.x == 0 && part) part[blockIdx.x] = t;
}

// --------------------------------------------------- preconditioner parts
// z_s = Z_s (w_s .* r_s) and partial coarse residual Phi_s^T (w_s .* r_s)
// (the dual basis Phi_dual for a general matrix, dd_phisi_dual_apply,
// module_dd.f90:6126-6206; oPhid = oPhi for symmetric matrices).
//
// With FP32 blocks (mixed precision) the blocks are exact FP32 numbers and the
// products are formed to FP64 accuracy: w .* r is kept as a double-float pair
// and each row sum is accumulated with error-free transformations.  The
// preconditioner is then a fixed linear operator (the FP32 blocks) applied
// without rounding noise: a product rounded to FP32 would add a relative
// perturbation of ~1e-7 at every application, which delays the convergence of
// the outer PCG on ill-conditioned problems (finite-precision CG behaves as if
// its operator's eigenvalues were smeared by the size of such perturbations).
template <typename T>
struct PcVec {
  using type = double;
};
template <>
struct PcVec<float> {
  using type = float2;  // (hi, lo) of an FP64 value
};

template <typename T>
__global__ void __launch_bounds__(AT) k_pc_local(const DevSub* __restrict__ ds, const T* __restrict__ pcpool,
                                                 const double* __restrict__ r, const int* __restrict__ uniq,
                                                 const double* __restrict__ wrep, double* __restrict__ zrep,
                                                 double* __restrict__ rcpart, int nrb, int ncpmax,
                                                 const PcgCtl* __restrict__ ctl) {
  if (ctl && ctl->done) return;
  const DevSub s = ds[blockIdx.y];
  const int r0 = blockIdx.x * AROWS;
  if (r0 >= s.ni) return;
  using V = typename PcVec<T>::type;
  extern __shared__ __align__(16) unsigned char smraw[];
  V* aux = reinterpret_cast<V*>(smraw);
  for (int j = threadIdx.x; j < s.NI; j += AT) {
    const double x = j < s.ni ? wrep[s.rep + j] * r[uniq[s.rep + j]] : 0.0;
    if constexpr (std::is_same_v<T, float>) {
      const float hi = (float)x;
      aux[j] = make_float2(hi, (float)(x - (double)hi));
    } else {
      aux[j] = x;
    }
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rend = min(r0 + AROWS, s.ni);
  for (int rr = r0 + warp; rr < rend; rr += AT / 32) {
    const T* row = pcpool + s.oZ + (long long)rr * s.NI;
    if constexpr (std::is_same_v<T, float>) {
      dfacc acc;
      for (int j = lane; j < s.NI; j += 32) {
        const float z = __ldg(row + j);
        const float2 x = aux[j];
        acc.fma_df(dfloat{x.x, x.y}, z);
      }
      for (int o = 16; o > 0; o >>= 1) {
        dfacc other;
        other.s = __shfl_xor_sync(0xffffffffu, acc.s, o);
        other.c = __shfl_xor_sync(0xffffffffu, acc.c, o);
        acc.merge(other);
      }
      if (lane == 0) zrep[s.rep + rr] = acc.to_double();
    } else {
      T acc = T(0);
      for (int j = lane; j < s.NI; j += 32) acc += __ldg(row + j) * aux[j];
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
      if (lane == 0) zrep[s.rep + rr] = (double)acc;
    }
  }
  // coarse residual partial over this CTA's rows
  for (int c = threadIdx.x; c < s.nc; c += AT) {
    double t = 0.0;
    for (int rr = r0; rr < rend; ++rr) {
      double x;
      if constexpr (std::is_same_v<T, float>) x = (double)aux[rr].x + (double)aux[rr].y;
      else x = aux[rr];
      t += (double)pcpool[s.oPhid + (long long)rr * s.ncp + c] * x;
    }
    rcpart[((long long)blockIdx.y * nrb + blockIdx.x) * ncpmax + c] = t;
  }
}

// r_c[q] = sum over the subdomain constraints mapped to coarse dof q
// (also as a double-float pair in rdf when given, the operand of k_coarse_gemv<float>)
__global__ void k_coarse_gather(int ndofc, const int* __restrict__ cptr, const int* __restrict__ csub,
                                const int* __restrict__ cloc, const DevSub* __restrict__ ds,
                                const double* __restrict__ rcpart, int nrb, int ncpmax, double* __restrict__ rc,
                                const PcgCtl* __restrict__ ctl, float2* __restrict__ rdf = nullptr) {
  if (ctl && ctl->done) return;
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= ndofc) return;
  double t = 0.0;
  for (int e = cptr[q]; e < cptr[q + 1]; ++e) {
    int s = csub[e], c = cloc[e];
    int nb = (ds[s].ni + AROWS - 1) / AROWS;
    for (int b = 0; b < nb; ++b) t += rcpart[((long long)s * nrb + b) * ncpmax + c];
  }
  rc[q] = t;
  if (rdf) {
    const dfloat v = df_from_double(t);
    rdf[q] = make_float2(v.hi, v.lo);
  }
}

// Coarse solve u_c = Ac^-1 r_c by an explicit inverse M of the coarse matrix
// (factor precision) with FP64 refinement against the FP64 coarse matrix:
//   u = M r;  repeat: u += M (r - Ac u).
// mode 0: u = M v;  mode 1: u += M v  (warp per row, FP64 accumulation)
// With an FP32 inverse the products M_ij v_j are formed exactly on the FP32
// pipes, with v given as double-float pairs (vdf, written by the kernel that
// produced v) and error-free sums, instead of in FP64, whose rate on this
// part is a small fraction of FP32.
template <typename T>
__global__ void __launch_bounds__(256) k_coarse_gemv(int n, int ld, const T* __restrict__ m,
                                                     const double* __restrict__ v, const float2* __restrict__ vdf,
                                                     double* __restrict__ u, int mode,
                                                     const PcgCtl* __restrict__ ctl) {
  if (ctl && ctl->done) return;
  int row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= n) return;
  const T* a = m + (long long)row * ld;
  double t;
  if constexpr (std::is_same_v<T, float>) {
    dfacc acc;
#pragma unroll 4
    for (int j = lane; j < n; j += 32) {
      const float2 x = __ldg(vdf + j);
      acc.fma_df(dfloat{x.x, x.y}, __ldg(a + j));
    }
    for (int o = 16; o > 0; o >>= 1) {
      dfacc other;
      other.s = __shfl_xor_sync(0xffffffffu, acc.s, o);
      other.c = __shfl_xor_sync(0xffffffffu, acc.c, o);
      acc.merge(other);
    }
    t = acc.to_double();
  } else {
    t = 0.0;
    for (int j = lane; j < n; j += 32) t += (double)a[j] * v[j];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  }
  if (lane == 0) u[row] = mode ? u[row] + t : t;
}

// res = r - Ac u with the sparse FP64 coarse matrix
__global__ void k_coarse_residual(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                  const double* __restrict__ val, const double* __restrict__ r,
                                  const double* __restrict__ u, double* __restrict__ res,
                                  const PcgCtl* __restrict__ ctl, float2* __restrict__ rdf = nullptr) {
  if (ctl && ctl->done) return;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double t = r[i];
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) t -= val[q] * u[col[q]];
  res[i] = t;
  if (rdf) {
    const dfloat v = df_from_double(t);
    rdf[i] = make_float2(v.hi, v.lo);
  }
}

// deterministic assembly of the coarse matrix: every nonzero sums its
// subdomain contributions in a fixed order (levels_prepare_last_level,
// module_levels.f90:3075-3090); the lower part is also written, in factor
// precision, into the dense block layout that the factor kernels use
template <typename T>
__global__ void k_coarse_assemble(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                  const int* __restrict__ cptr, const long long* __restrict__ contrib,
                                  const double* __restrict__ small, double* __restrict__ val, T* __restrict__ fpool,
                                  BandDesc d, const BandDesc* __restrict__ du) {
  int i = blockIdx.x;
  if (i >= n) return;
  for (int q = ptr[i] + threadIdx.x; q < ptr[i + 1]; q += blockDim.x) {
    double t = 0.0;
    for (int e = cptr[q]; e < cptr[q + 1]; ++e) t += small[contrib[e]];
    val[q] = t;
    int j = col[q];
    if (du) lu_slot<T>(d, *du, fpool, i, j) = T(t);  // general: L and U^T bands
    else if (j <= i) fpool[band_block(d, i / NB, j / NB) + (i % NB) * NB + j % NB] = T(t);
  }
}

template <typename T>
__global__ void k_coarse_pad(int n, int ld, T* __restrict__ fpool, BandDesc d) {
  int i = n + blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ld) fpool[band_block(d, i / NB, i / NB) + (i % NB) * NB + i % NB] = T(1);
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < ld) fpool[d.oB + (long long)k * ld + k] = T(1);  // identity right-hand side
}

// zw[rep + i] = w_i (z_s[i] + Phi_s[i, :] u_c|_s) for the interface rows of
// every subdomain (the subdomain part of levels_add_first_level,
// module_levels.f90:4252-4346); k_assemble_dot then sums them per unique dof.
// grid (row tiles of ZP_ROWS, nsub); the tile of Phi (contiguous rows) is
// staged through shared memory with coalesced loads, rows padded by one word.
// With FP32 Phi the products are exact double-float sums on the FP32 pipes.
constexpr int ZP_ROWS = 128;
template <typename T>
__global__ void __launch_bounds__(ZP_ROWS) k_zphi(const DevSub* __restrict__ ds, const T* __restrict__ pcpool,
                                                  const double* __restrict__ zrep, const double* __restrict__ wrep,
                                                  const int* __restrict__ cmap, const double* __restrict__ uc,
                                                  double* __restrict__ zw, const PcgCtl* __restrict__ ctl) {
  if (ctl && ctl->done) return;
  const DevSub s = ds[blockIdx.y];
  const int r0 = blockIdx.x * ZP_ROWS;
  if (r0 >= s.ni) return;
  using V = typename PcVec<T>::type;
  extern __shared__ __align__(16) unsigned char zp_raw[];
  V* us = reinterpret_cast<V*>(zp_raw);                  // u_c at the subdomain's constraints
  T* tile = reinterpret_cast<T*>(us + s.ncp);             // rows x (ncp + 1)
  const int nc = uc ? s.nc : 0, ldt = s.ncp + 1;
  const int rows = min(ZP_ROWS, s.ni - r0);
  for (int c = threadIdx.x; c < nc; c += ZP_ROWS) {
    const double x = uc[cmap[s.coff + c]];
    if constexpr (std::is_same_v<T, float>) {
      const float hi = (float)x;
      us[c] = make_float2(hi, (float)(x - (double)hi));
    } else {
      us[c] = x;
    }
  }
  if (nc > 0) {
    const T* src = pcpool + s.oPhi + (long long)r0 * s.ncp;
    for (int e = threadIdx.x; e < rows * s.ncp; e += ZP_ROWS) tile[(e / s.ncp) * ldt + e % s.ncp] = __ldg(src + e);
  }
  __syncthreads();
  const int r = threadIdx.x;
  if (r >= rows) return;
  const T* ph = tile + r * ldt;
  double t;
  if constexpr (std::is_same_v<T, float>) {
    dfacc acc;
    for (int c = 0; c < nc; ++c) acc.fma_df(dfloat{us[c].x, us[c].y}, ph[c]);
    t = acc.to_double();
  } else {
    t = 0.0;
    for (int c = 0; c < nc; ++c) t += ph[c] * us[c];
  }
  const long long o = (long long)s.rep + r0 + r;
  zw[o] = wrep[o] * (zrep[o] + t);
}

// z[g] = sum_s w_s (z_s + Phi_s u_c|_s); partial (r, z)
template <typename T>
__global__ void __launch_bounds__(RT) k_assemble_z(int n, Owners own, const DevSub* __restrict__ ds,
                                                   const T* __restrict__ pcpool, const double* __restrict__ zrep,
                                                   const double* __restrict__ wrep, const int* __restrict__ cmap,
                                                   const double* __restrict__ uc, const double* __restrict__ wsum,
                                                   const double* __restrict__ r, double* __restrict__ z,
                                                   double* __restrict__ part, const PcgCtl* __restrict__ ctl) {
  if (ctl && ctl->done) return;
  __shared__ double sh[32];
  double loc = 0.0;
  for (int g = blockIdx.x * RT + threadIdx.x; g < n; g += gridDim.x * RT) {
    double v = 0.0;
    for (int q = own.ptr[g]; q < own.ptr[g + 1]; ++q) {
      int sidx = own.sub[q], i = own.loc[q];
      const DevSub& s = ds[sidx];
      double t = zrep[s.rep + i];
      const T* ph = pcpool + s.oPhi + (long long)i * s.ncp;
      for (int c = 0; c < s.nc; ++c) t += (double)ph[c] * uc[cmap[s.coff + c]];
      v += wrep[s.rep + i] * t;
    }
    z[g] = v;
    loc += wsum[g] * r[g] * v;
  }
  double t = block_reduce(loc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// ---------------------------------------------------------------- scalars
__device__ __forceinline__ double sum_parts(const double* part, int n, double* sh) {
  double v = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[i];
  return block_reduce(v, sh);
}

// pap and alpha = rmp / pap  (module_krylov.f90:637-726)
__global__ void k_sc_alpha(PcgCtl* ctl, const double* __restrict__ part, int npart) {
  if (ctl->done) return;
  __shared__ double sh[32];
  double pap = sum_parts(part, npart, sh);
  if (threadIdx.x == 0) {
    ctl->pap = pap;
    if (!(pap > 0.0)) ctl->warn |= 1;
    ctl->alpha = ctl->rmp / pap;
  }
}

// x += alpha p, r -= alpha ap; partial (r, r)
__global__ void __launch_bounds__(RT) k_update_xr(int n, const PcgCtl* __restrict__ ctl, double* __restrict__ x,
                                                  double* __restrict__ r, const double* __restrict__ p,
                                                  const double* __restrict__ ap, const double* __restrict__ wsum,
                                                  double* __restrict__ part) {
  if (ctl->done) return;
  __shared__ double sh[32];
  const double alpha = ctl->alpha;
  double loc = 0.0;
  for (int g = blockIdx.x * RT + threadIdx.x; g < n; g += gridDim.x * RT) {
    x[g] += alpha * p[g];
    double rv = r[g] - alpha * ap[g];
    r[g] = rv;
    loc += wsum[g] * rv * rv;
  }
  double t = block_reduce(loc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// residual norm and the stop tests of module_krylov.f90:744-810
__global__ void k_sc_res(PcgCtl* ctl, const double* __restrict__ part, int npart, double* __restrict__ hist) {
  if (ctl->done) return;
  __shared__ double sh[32];
  double nr2 = sum_parts(part, npart, sh);
  if (threadIdx.x == 0) {
    int iter = ctl->iter;
    ctl->normres2 = nr2;
    double relres = sqrt(nr2) / ctl->normres0;
    ctl->relres = relres;
    hist[iter - 1] = relres;
    if (relres < ctl->tol) {
      ctl->done = 1; ctl->reason = 0; ctl->num_iter = iter; ctl->nw = iter - 1;
    } else if (iter == ctl->maxit) {
      ctl->done = 1; ctl->reason = -1; ctl->num_iter = iter; ctl->nw = iter - 1;
    } else {
      if (relres < ctl->lastres) ctl->ndecr = 0;
      else {
        ctl->ndecr += 1;
        if (ctl->ndecr >= ctl->ndecrmax) { ctl->done = 1; ctl->reason = -2; ctl->num_iter = iter; ctl->nw = iter - 1; }
      }
      ctl->lastres = relres;
    }
  }
}

// rmp, beta and the Lanczos tridiagonal (module_krylov.f90:841-886)
__global__ void k_sc_beta(PcgCtl* ctl, const double* __restrict__ part, int npart, double* __restrict__ diag,
                          double* __restrict__ subdiag) {
  if (ctl->done) return;
  __shared__ double sh[32];
  double rmp = sum_parts(part, npart, sh);
  if (threadIdx.x == 0) {
    if (!(rmp > 0.0)) ctl->warn |= 2;
    double beta = rmp / ctl->rmp;
    ctl->beta = beta;
    ctl->rmp = rmp;
    int iter = ctl->iter;
    double alpha = ctl->alpha;
    diag[iter - 1] += 1.0 / alpha;
    diag[iter] = beta / alpha;
    subdiag[iter - 1] = beta >= 0.0 ? -sqrt(beta) / alpha : 0.0;
    ctl->iter = iter + 1;
  }
}

__global__ void __launch_bounds__(RT) k_update_p(int n, const PcgCtl* __restrict__ ctl, double* __restrict__ p,
                                                 const double* __restrict__ z) {
  if (ctl->done) return;
  const double beta = ctl->beta;
  for (int g = blockIdx.x * RT + threadIdx.x; g < n; g += gridDim.x * RT) p[g] = z[g] + beta * p[g];
}

// ------------------------------------------------------- Krylov recycling
// Stored S-orthonormal search directions V (n x cap, column-major) and
// W = S V, nact of them in use (module_krylov.f90:33-43, 663-726).  Kernels
// with a control block do nothing once the iteration has stopped.

// partial weighted dots (basis_j, v)_w for j < nact: part[block * cap + j]
__global__ void __launch_bounds__(RT) k_rc_dots(int n, int cap, const int* __restrict__ nact,
                                                const double* __restrict__ basis, const double* __restrict__ wsum,
                                                const double* __restrict__ v, double* __restrict__ part,
                                                const PcgCtl* __restrict__ ctl) {
  if (ctl && ctl->done) return;
  __shared__ double sh[32];
  const int na = *nact;
  for (int j = 0; j < na; ++j) {
    const double* b = basis + (long long)j * n;
    double loc = 0.0;
    for (int g = blockIdx.x * RT + threadIdx.x; g < n; g += gridDim.x * RT) loc += wsum[g] * b[g] * v[g];
    const double t = block_reduce(loc, sh);
    if (threadIdx.x == 0) part[blockIdx.x * cap + j] = t;
  }
}

__global__ void k_rc_coef(int cap, const int* __restrict__ nact, const double* __restrict__ part, int npart,
                          double* __restrict__ coef, const PcgCtl* __restrict__ ctl) {
  if (ctl && ctl->done) return;
  const int na = *nact;
  for (int j = threadIdx.x; j < na; j += blockDim.x) {
    double t = 0.0;
    for (int b = 0; b < npart; ++b) t += part[b * cap + j];
    coef[j] = t;
  }
}

// v += sign * V coef
__global__ void __launch_bounds__(RT) k_rc_combine(int n, const int* __restrict__ nact, const double* __restrict__ V,
                                                   const double* __restrict__ coef, double sign, double* __restrict__ v,
                                                   const PcgCtl* __restrict__ ctl) {
  if (ctl && ctl->done) return;
  const int na = *nact;
  for (int g = blockIdx.x * RT + threadIdx.x; g < n; g += gridDim.x * RT) {
    double t = 0.0;
    for (int j = 0; j < na; ++j) t += V[(long long)j * n + g] * coef[j];
    v[g] += sign * t;
  }
}

// V(:, nact) = p / sqrt(pap), W(:, nact) = ap / sqrt(pap) while there is room
__global__ void __launch_bounds__(RT) k_rc_store(int n, int cap, const int* __restrict__ nact,
                                                 const double* __restrict__ p, const double* __restrict__ ap,
                                                 double* __restrict__ V, double* __restrict__ W,
                                                 const PcgCtl* __restrict__ ctl) {
  if (ctl->done) return;
  const int na = *nact;
  if (na >= cap) return;
  const double sc = 1.0 / sqrt(ctl->pap);
  for (int g = blockIdx.x * RT + threadIdx.x; g < n; g += gridDim.x * RT) {
    V[(long long)na * n + g] = sc * p[g];
    W[(long long)na * n + g] = sc * ap[g];
  }
}

__global__ void k_rc_bump(int cap, int* __restrict__ nact, const PcgCtl* __restrict__ ctl) {
  if (ctl->done) return;
  if (*nact < cap) *nact += 1;
}

// -------------------------------------------------------- helper kernels
// v[g] = sum over holders of a replicated vector (reduced rhs assembly)
__global__ void k_assemble_plain(int n, Owners own, const double* __restrict__ rep, const int* __restrict__ fixed,
                                 double* __restrict__ out) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  double v = 0.0;
  for (int q = own.ptr[g]; q < own.ptr[g + 1]; ++q) v += rep[own.rep[q]];
  if (fixed && fixed[g]) v = 0.0;
  out[g] = v;
}

// weighted dot product partials (a, b)_w
__global__ void __launch_bounds__(RT) k_dot(int n, const double* __restrict__ a, const double* __restrict__ b,
                                            const double* __restrict__ wsum, double* __restrict__ part) {
  __shared__ double sh[32];
  double loc = 0.0;
  for (int g = blockIdx.x * RT + threadIdx.x; g < n; g += gridDim.x * RT) loc += wsum[g] * a[g] * b[g];
  double t = block_reduce(loc, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void k_sum_parts(const double* __restrict__ part, int npart, double* __restrict__ out) {
  __shared__ double sh[32];
  double v = sum_parts(part, npart, sh);
  if (threadIdx.x == 0) *out = v;
}

__global__ void k_axpy(int n, double a, const double* __restrict__ x, double* __restrict__ y) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n) y[g] += a * x[g];
}

// y = a x + b y
__global__ void k_axpby(int n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n) y[g] = a * x[g] + b * y[g];
}

// v = 0 at the fixed interface dofs (dd_fix_bc_interface_dual, module_dd.f90:3468-3505)
__global__ void k_zero_fixed(int n, const int* __restrict__ fixed, double* __restrict__ v) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n && fixed[g]) v[g] = 0.0;
}

// interior values u_o = v - X(:, 0:ni) x_s  (module_dd.f90:6811-6932): 64
// rows per CTA, the gathered interface solution staged once in shared memory
// as double-float, X read as its double-float pair
constexpr int POST_ROWS = 64;
__global__ void __launch_bounds__(256) k_post_df(const DevSub* __restrict__ ds, const float* __restrict__ pool,
                                                 const double* __restrict__ x, const int* __restrict__ uniq,
                                                 double* __restrict__ uo, const long long* __restrict__ uo_off) {
  const DevSub s = ds[blockIdx.y];
  const int r0 = blockIdx.x * POST_ROWS;
  if (r0 >= s.no) return;
  extern __shared__ __align__(16) unsigned char smraw[];
  float2* xs = reinterpret_cast<float2*>(smraw);
  for (int j = threadIdx.x; j <= s.ni; j += blockDim.x) {
    dfloat v = j < s.ni ? df_from_double(-x[uniq[s.rep + j]]) : dfloat{1.f, 0.f};
    xs[j] = make_float2(v.hi, v.lo);
  }
  __syncthreads();
  const long long comp = (long long)s.NO * s.NR;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rend = min(r0 + POST_ROWS, s.no);
  for (int row = r0 + warp; row < rend; row += 8) {
    const float* X0 = pool + s.oXc + (long long)row * s.NR;
    const float* X1 = X0 + comp;
    dfacc acc;
    for (int j = lane; j <= s.ni; j += 32) {
      float2 xv = xs[j];
      acc.fma_df(dfloat{xv.x, xv.y}, dfloat{X0[j], X1[j]});
    }
    for (int o = 16; o > 0; o >>= 1) {
      dfacc other;
      other.s = __shfl_xor_sync(0xffffffffu, acc.s, o);
      other.c = __shfl_xor_sync(0xffffffffu, acc.c, o);
      acc.merge(other);
    }
    if (lane == 0) uo[uo_off[blockIdx.y] + row] = acc.to_double();
  }
}

__global__ void __launch_bounds__(256) k_post_f64(const DevSub* __restrict__ ds, const double* __restrict__ pool,
                                                  const double* __restrict__ x, const int* __restrict__ uniq,
                                                  double* __restrict__ uo, const long long* __restrict__ uo_off) {
  const DevSub s = ds[blockIdx.y];
  int row = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (row >= s.no) return;
  const double* X = pool + s.oXc + (long long)row * s.NR;
  double acc = 0.0;
  for (int j = lane; j < s.ni; j += 32) acc -= X[j] * x[uniq[s.rep + j]];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) uo[uo_off[blockIdx.y] + row] = acc + X[s.ni];
}

}  // namespace bddc
