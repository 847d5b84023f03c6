// Double-float (pair of FP32) arithmetic for FP64-accurate products on the
// FP32 pipes.  GB300 runs FP64 at a small fraction of its FP32 rate, so the
// FP64-accurate parts of the hot path (the Schur operator apply and the
// residuals of the interior-solve refinement) keep 2 x FP32 values per number
// and use error-free transformations (Knuth's two-sum, FMA-based two-product;
// Dekker 1971) instead of FP64 instructions.
#pragma once

#include <cuda_runtime.h>

namespace bddc {

struct dfloat {
  float hi, lo;
};

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// accumulator: (s, c) with value s + c; c collects the low-order parts
struct dfacc {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float p) {  // exact addition of one FP32 value
    float t, e;
    two_sum(s, p, t, e);
    s = t;
    c += e;
  }
  // += a * x with a, x double-float (a.lo*x.lo dropped, relative 2^-48 when x
  // is normalised, |x.lo| <= 2^-24 |x.hi|)
  __device__ __forceinline__ void fma_df(dfloat a, dfloat x) {
    float p = a.hi * x.hi;
    float e = fmaf(a.hi, x.hi, -p);
    e = fmaf(a.hi, x.lo, e);
    e = fmaf(a.lo, x.hi, e);
    add(p);
    c += e;
  }
  // += a * x with a double-float, x an exact FP32 value
  __device__ __forceinline__ void fma_df(dfloat a, float x) {
    float p = a.hi * x;
    float e = fmaf(a.hi, x, -p);
    e = fmaf(a.lo, x, e);
    add(p);
    c += e;
  }
  __device__ __forceinline__ void add_df(dfloat v) {
    add(v.hi);
    c += v.lo;
  }
  __device__ __forceinline__ void merge(const dfacc& o) {
    add(o.s);
    c += o.c;
  }
  __device__ __forceinline__ dfloat value() const {
    dfloat r;
    r.hi = s + c;
    r.lo = c - (r.hi - s);
    return r;
  }
  __device__ __forceinline__ double to_double() const { return (double)s + (double)c; }
};

// One multiply-add of a double-float product a * b (a = ah + al,
// b = bh + bl) into the unevaluated sum (sh, sl): the exact product ah bh (a
// rounded product and its fma error) plus the cross terms ah bl + al bh,
// accumulated with an error-free two-sum.  Accuracy about 2^-44 relative to
// sum |a b|, FP64-like for these products.
__device__ __forceinline__ void df_mac(float& sh, float& sl, float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  const float e = __fmaf_rn(ah, bh, -p);
  const float c = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, e));
  const float t = __fadd_rn(sh, p);
  const float bp = __fsub_rn(t, sh);
  const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  sh = t;
  sl = __fadd_rn(sl, __fadd_rn(err, c));
}

__device__ __forceinline__ dfloat df_from_double(double v) {
  dfloat r;
  r.hi = (float)v;
  r.lo = (float)(v - (double)r.hi);
  return r;
}

__device__ __forceinline__ double df_to_double(dfloat v) { return (double)v.hi + (double)v.lo; }

}  // namespace bddc
