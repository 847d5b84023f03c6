// Per-element gradient of an objective J(u) with respect to element
// coefficients kappa_e of K(kappa) = sum_e kappa_e K_e^0:
//     dJ/dkappa_e = - lambda_e^T K_e^0 u_e,
// with u the solution and lambda the adjoint solution (K lambda = dJ/du, the
// same SPD operator).  Element vectors are gathered from the global vectors
// here rather than stored.  Entry point: bddcml_element_gradient_dev_c.
#include <string>

#include <cuda_runtime.h>

#include "bddc_internal.hpp"

namespace bddc {

namespace {

constexpr int GRAD_MAX_NNE = 27;  // nodes of a Q2 hexahedron, the largest element handled
constexpr int GRAD_THREADS = 128;

__global__ void __launch_bounds__(GRAD_THREADS) k_element_gradient(int nelem, int nne, const int* __restrict__ inet,
                                                                   const double* __restrict__ ke0, long long kstride,
                                                                   const double* __restrict__ u,
                                                                   const double* __restrict__ lam,
                                                                   double* __restrict__ grad) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nelem) return;
  const int* ie = inet + (long long)e * nne;
  const double* K = ke0 + (long long)e * kstride;
  double ue[GRAD_MAX_NNE], le[GRAD_MAX_NNE];
  for (int a = 0; a < nne; ++a) {
    const int g = ie[a];
    ue[a] = u[g];
    le[a] = lam[g];
  }
  double s = 0.0;
  for (int a = 0; a < nne; ++a) {
    double t = 0.0;
    for (int b = 0; b < nne; ++b) t += __ldg(K + a * nne + b) * ue[b];
    s += le[a] * t;
  }
  grad[e] = -s;
}

}  // namespace

bool device_element_gradient(int nelem, int nne, const int* inet, const double* ke0, bool per_element,
                             const double* u, const double* lam, double* grad, Error& err) {
  if (nelem < 0 || nne <= 0 || nne > GRAD_MAX_NNE) {
    err = Error{ERR_ARGUMENT, "element node count must be in 1.." + std::to_string(GRAD_MAX_NNE)};
    return false;
  }
  if (nelem == 0) return true;
  if (!inet || !ke0 || !u || !lam || !grad) {
    err = Error{ERR_ARGUMENT, "null device pointer"};
    return false;
  }
  const long long kstride = per_element ? (long long)nne * nne : 0;
  k_element_gradient<<<(nelem + GRAD_THREADS - 1) / GRAD_THREADS, GRAD_THREADS>>>(nelem, nne, inet, ke0, kstride, u,
                                                                                  lam, grad);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) {
    err = Error{ERR_CUDA, std::string("element gradient kernel: ") + cudaGetErrorString(e)};
    return false;
  }
  return true;
}

}  // namespace bddc
