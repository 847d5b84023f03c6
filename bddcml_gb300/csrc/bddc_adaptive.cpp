// Adaptive face constraints, host part: the face pairs and their operators
// (adaptivity_solve_eigenvectors, module_adaptivity.f90:296-2514) and the
// loading of the selected eigenvectors as face constraints
// (dd_load_adaptive_constraints + dd_orthogonalize_constraints,
// module_dd.f90:4386-4760).  The eigenproblems themselves run on the GPU
// (device_setup, bddc_device.cu).
#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <string>
#include <unordered_map>

#include "bddc_internal.hpp"

namespace bddc {

namespace {

// cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major,
// overwritten); eigenvalues in w, eigenvectors in the columns of z
void jacobi_eig(int n, vector<double>& a, vector<double>& w, vector<double>& z) {
  z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) z[(size_t)i * n + i] = 1.0;
  for (int sweep = 0; sweep < 50; ++sweep) {
    double off = 0.0, dg = 0.0;
    for (int r = 0; r < n; ++r)
      for (int c = 0; c < n; ++c) (r == c ? dg : off) += a[(size_t)r * n + c] * a[(size_t)r * n + c];
    if (off <= 1e-30 * dg || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[(size_t)p * n + q];
        if (apq == 0.0) continue;
        const double th = (a[(size_t)q * n + q] - a[(size_t)p * n + p]) / (2.0 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), sn = t * c;
        for (int j = 0; j < n; ++j) {
          const double xp = a[(size_t)p * n + j], xq = a[(size_t)q * n + j];
          a[(size_t)p * n + j] = c * xp - sn * xq;
          a[(size_t)q * n + j] = sn * xp + c * xq;
        }
        for (int j = 0; j < n; ++j) {
          const double xp = a[(size_t)j * n + p], xq = a[(size_t)j * n + q];
          a[(size_t)j * n + p] = c * xp - sn * xq;
          a[(size_t)j * n + q] = sn * xp + c * xq;
          const double zp = z[(size_t)j * n + p], zq = z[(size_t)j * n + q];
          z[(size_t)j * n + p] = c * zp - sn * zq;
          z[(size_t)j * n + q] = sn * zp + c * zq;
        }
        a[(size_t)p * n + q] = a[(size_t)q * n + p] = 0.0;
      }
  }
  w.resize(n);
  for (int i = 0; i < n; ++i) w[i] = a[(size_t)i * n + i];
}

}  // namespace

vector<double> host_coarse_null_coefficients(int nc, int ld, const double* ac, int& d) {
  vector<double> a((size_t)nc * nc), w, z;
  for (int r = 0; r < nc; ++r)
    for (int c = 0; c < nc; ++c) a[(size_t)r * nc + c] = 0.5 * (ac[(size_t)r * ld + c] + ac[(size_t)c * ld + r]);
  jacobi_eig(nc, a, w, z);
  double wmax = 0.0;
  for (double x : w) wmax = std::max(wmax, std::fabs(x));
  vector<double> y;
  d = 0;
  // the tolerance of Octave's null() relaxed as in module_adaptivity.f90:1485-1489
  // (n * max eigenvalue * 4 eps), with the 2^-44 accuracy of the products
  const double tol = std::max(1, nc) * wmax * 4.0 * 5.7e-14;
  for (int k = 0; k < nc; ++k)
    if (std::fabs(w[k]) <= tol) {
      for (int r = 0; r < nc; ++r) y.push_back(z[(size_t)r * nc + k]);
      ++d;
    }
  return y;
}

void host_adaptive_pairs(const Solver& S, AdaptivePairs& P, const vector<vector<double>>& nulls) {
  const int nsub = (int)S.subs.size();
  // pairs = faces, in the order of their global coarse node (dd_create_pairs,
  // module_dd.f90:10785-11008)
  std::map<int, vector<std::pair<int, int>>> faces;
  for (int t = 0; t < nsub; ++t)
    for (int c = 0; c < (int)S.subs[t].cnodes.size(); ++c)
      if (S.subs[t].cnodes[c].itype == 1) faces[S.subs[t].cnodes[c].global_number].push_back({t, c});
  P = AdaptivePairs{};
  for (auto& f : faces) {
    if (f.second.size() != 2) throw Error{ERR_NUMERIC, "a face not shared by exactly two subdomains"};
    P.si.push_back(f.second[0].first);
    P.fi.push_back(f.second[0].second);
    P.sj.push_back(f.second[1].first);
    P.fj.push_back(f.second[1].second);
  }
  const int np = (int)P.si.size();
  P.npair = np;
  P.ni.resize(np); P.n.resize(np); P.m.resize(np); P.k.resize(np); P.md.resize(np);
  vector<vector<int>> ca(np), cb(np);
  vector<vector<double>> wa(np), wb(np), q(np);
#pragma omp parallel for schedule(dynamic)
  for (int p = 0; p < np; ++p) {
    const Subdomain& A = S.subs[P.si[p]];
    const Subdomain& B = S.subs[P.sj[p]];
    const int ni = A.ndofi, n = ni + B.ndofi;
    P.ni[p] = ni;
    P.n[p] = n;
    // dofs on interface nodes of both subdomains, weighted by rho / (rho_a + rho_b)
    std::unordered_map<int, int> jnode;
    for (int i = 0; i < B.nnodi; ++i) jnode.emplace(B.isngn[B.iin[i]], i);
    for (int i = 0; i < A.nnodi; ++i) {
      auto it = jnode.find(A.isngn[A.iin[i]]);
      if (it == jnode.end()) continue;
      const int nd = A.nndf[A.iin[i]];
      for (int d = 0; d < nd; ++d) {
        const int a = A.kdofi[i] + d, b = B.kdofi[it->second] + d;
        const double ra = A.rhoi[a], rb = B.rhoi[b];
        ca[p].push_back(a);
        cb[p].push_back(ni + b);
        wa[p].push_back(ra / (ra + rb));
        wb[p].push_back(rb / (ra + rb));
      }
    }
    // D^T = [C_i; -C_j] on the coarse dofs both subdomains carry; orthonormal
    // basis of its range by Gram-Schmidt, twice
    std::unordered_map<int, int> jrow;
    for (int r = 0; r < B.nconstr; ++r) jrow.emplace(B.indrowc[r], r);
    int m = 0;
    vector<double> v(n);
    for (int r = 0; r < A.nconstr; ++r) {
      auto it = jrow.find(A.indrowc[r]);
      if (it == jrow.end()) continue;
      std::fill(v.begin(), v.end(), 0.0);
      for (int e = A.c_ptr[r]; e < A.c_ptr[r + 1]; ++e) v[A.c_col[e]] += A.c_val[e];
      for (int e = B.c_ptr[it->second]; e < B.c_ptr[it->second + 1]; ++e) v[ni + B.c_col[e]] -= B.c_val[e];
      for (int pass = 0; pass < 2; ++pass)
        for (int c = 0; c < m; ++c) {
          const double* qc = &q[p][(size_t)c * n];
          double t = 0.0;
          for (int i = 0; i < n; ++i) t += qc[i] * v[i];
          for (int i = 0; i < n; ++i) v[i] -= t * qc[i];
        }
      double nv = 0.0;
      for (double x : v) nv += x * x;
      nv = std::sqrt(nv);
      if (nv < 1e-12) continue;
      for (double x : v) q[p].push_back(x / nv);
      ++m;
    }
    const int mD = m;
    // null(S) within null(D): from the subdomains' null spaces N = diag(N_i, N_j),
    // the combinations y with Q^T N y = 0; appended to Q so that the search
    // space excludes them (the projection of adaptivity_apply_complementary_projection,
    // module_adaptivity.f90:3026-3065)
    const int di = (int)(nulls[P.si[p]].size() / std::max(1, ni));
    const int dj = (int)(nulls[P.sj[p]].size() / std::max(1, B.ndofi));
    const int d = di + dj;
    if (d > 0) {
      vector<double> N((size_t)n * d, 0.0);
      for (int c = 0; c < di; ++c)
        for (int r = 0; r < ni; ++r) N[(size_t)c * n + r] = nulls[P.si[p]][(size_t)c * ni + r];
      for (int c = 0; c < dj; ++c)
        for (int r = 0; r < B.ndofi; ++r) N[(size_t)(di + c) * n + ni + r] = nulls[P.sj[p]][(size_t)c * B.ndofi + r];
      // M = Q^T N (m x d); eigenvectors of M^T M with eigenvalue ~ 0
      vector<double> M((size_t)m * d, 0.0), mtm((size_t)d * d, 0.0), w, z;
      for (int a = 0; a < m; ++a)
        for (int c = 0; c < d; ++c) {
          double t = 0.0;
          for (int r = 0; r < n; ++r) t += q[p][(size_t)a * n + r] * N[(size_t)c * n + r];
          M[(size_t)a * d + c] = t;
        }
      for (int a = 0; a < d; ++a)
        for (int b = 0; b < d; ++b) {
          double t = 0.0;
          for (int r = 0; r < m; ++r) t += M[(size_t)r * d + a] * M[(size_t)r * d + b];
          mtm[(size_t)a * d + b] = t;
        }
      jacobi_eig(d, mtm, w, z);
      for (int k = 0; k < d; ++k) {
        if (w[k] > 1e-8) continue;
        for (int r = 0; r < n; ++r) {
          double t = 0.0;
          for (int c = 0; c < d; ++c) t += N[(size_t)c * n + r] * z[(size_t)c * d + k];
          v[r] = t;
        }
        for (int pass = 0; pass < 2; ++pass)
          for (int c = 0; c < m; ++c) {
            const double* qc = &q[p][(size_t)c * n];
            double t = 0.0;
            for (int i = 0; i < n; ++i) t += qc[i] * v[i];
            for (int i = 0; i < n; ++i) v[i] -= t * qc[i];
          }
        double nv = 0.0;
        for (double x : v) nv += x * x;
        nv = std::sqrt(nv);
        if (nv < 1e-6) continue;
        for (double x : v) q[p].push_back(x / nv);
        ++m;
      }
    }
    P.m[p] = m;
    P.md[p] = mD;
    P.k[p] = std::max(0, std::min(AdaptivePairs::KMAX, (int)ca[p].size() - mD));
  }
  P.vo.resize(np); P.qo.resize(np); P.cptr.assign(np + 1, 0);
  for (int p = 0; p < np; ++p) {
    P.vo[p] = P.nvec;
    P.nvec += (long long)P.n[p] * AdaptivePairs::KMAX;
    P.qo[p] = P.nq;
    P.nq += (long long)P.n[p] * P.m[p];
    P.cptr[p + 1] = P.cptr[p] + (int)ca[p].size();
    P.ca.insert(P.ca.end(), ca[p].begin(), ca[p].end());
    P.cb.insert(P.cb.end(), cb[p].begin(), cb[p].end());
    P.wa.insert(P.wa.end(), wa[p].begin(), wa[p].end());
    P.wb.insert(P.wb.end(), wb[p].begin(), wb[p].end());
    P.q.insert(P.q.end(), q[p].begin(), q[p].end());
  }
}

namespace {

// Orthonormal basis of the span of the ncol columns of m (nrow x ncol,
// column-major): Householder QR with column pivoting, keeping the leading
// columns whose |R_ii| is at least 1 % of |R_11| (DGEQP3 + DORGQR with the
// rule of dd_orthogonalize_constraints, module_dd.f90:4690-4733).
vector<double> orthonormal_rows(int nrow, int ncol, vector<double> m, int& nvalid) {
  const int kmax = std::min(nrow, ncol);
  vector<vector<double>> hv;
  vector<double> rd;
  for (int k = 0; k < kmax; ++k) {
    int best = k;
    double bn = -1.0;
    for (int c = k; c < ncol; ++c) {
      double t = 0.0;
      for (int r = k; r < nrow; ++r) t += m[(size_t)c * nrow + r] * m[(size_t)c * nrow + r];
      if (t > bn) { bn = t; best = c; }
    }
    if (best != k)
      for (int r = 0; r < nrow; ++r) std::swap(m[(size_t)k * nrow + r], m[(size_t)best * nrow + r]);
    const double nx = std::sqrt(std::max(0.0, bn));
    vector<double> v(nrow, 0.0);
    if (nx > 0.0) {
      const double alpha = m[(size_t)k * nrow + k] > 0 ? -nx : nx;
      for (int r = k; r < nrow; ++r) v[r] = m[(size_t)k * nrow + r];
      v[k] -= alpha;
      double nv = 0.0;
      for (int r = k; r < nrow; ++r) nv += v[r] * v[r];
      nv = std::sqrt(nv);
      if (nv > 0.0)
        for (int r = k; r < nrow; ++r) v[r] /= nv;
      for (int c = k; c < ncol; ++c) {
        double t = 0.0;
        for (int r = k; r < nrow; ++r) t += v[r] * m[(size_t)c * nrow + r];
        for (int r = k; r < nrow; ++r) m[(size_t)c * nrow + r] -= 2.0 * t * v[r];
      }
    }
    rd.push_back(m[(size_t)k * nrow + k]);
    hv.push_back(std::move(v));
  }
  nvalid = 0;
  if (kmax > 0 && std::fabs(rd[0]) > 1e-12) {
    for (int i = 0; i < kmax && std::fabs(rd[i]) >= 0.01 * std::fabs(rd[0]); ++i) nvalid = i + 1;
  }
  vector<double> qm((size_t)nrow * nvalid, 0.0);
  for (int c = 0; c < nvalid; ++c) {
    double* col = &qm[(size_t)c * nrow];
    col[c] = 1.0;
    for (int k = c; k >= 0; --k) {
      const auto& v = hv[k];
      double t = 0.0;
      for (int r = k; r < nrow; ++r) t += v[r] * col[r];
      for (int r = k; r < nrow; ++r) col[r] -= 2.0 * t * v[r];
    }
  }
  return qm;
}

// the arithmetic-average rows of a face (one row per dof component,
// module_dd.f90:4298-4384), ncdof x idofi.size()
vector<double> default_rows(const Subdomain& s, const CoarseNode& cn) {
  const int nv = (int)cn.idofi.size();
  vector<double> rows((size_t)cn.ncdof * nv, 0.0);
  int v = 0;
  for (int i : cn.inodi) {
    const int nd = s.nndf[s.iin[i]];
    for (int d = 0; d < nd; ++d, ++v)
      if (d < cn.ncdof) rows[(size_t)d * nv + v] = 1.0;
  }
  return rows;
}

}  // namespace

void host_load_adaptive(Solver& S, const AdaptivePairs& P, const vector<double>& eig, const vector<double>& cons) {
  const double tau = S.prm.adaptive_tau;
  for (double v : eig)
    if (!std::isfinite(v)) throw Error{ERR_NUMERIC, "adaptive constraints: non-finite eigenvalue"};
  for (double v : cons)
    if (!std::isfinite(v)) throw Error{ERR_NUMERIC, "adaptive constraints: non-finite constraint entry"};
  long long off = 0;
  int nadaptive = 0;
  for (int p = 0; p < P.npair; ++p) {
    Subdomain& A = S.subs[P.si[p]];
    Subdomain& B = S.subs[P.sj[p]];
    CoarseNode& ci = A.cnodes[P.fi[p]];
    CoarseNode& cj = B.cnodes[P.fj[p]];
    const int nv = (int)ci.idofi.size();
    if ((int)cj.idofi.size() != nv) throw Error{ERR_NUMERIC, "face with different dof counts in its two subdomains"};
    int nad = 0;
    for (int c = 0; c < P.k[p]; ++c)
      if (eig[(size_t)p * AdaptivePairs::KMAX + c] >= tau) ++nad;
    nadaptive += nad;
    // columns: the face's current rows, then the adaptive rows restricted to
    // the face dofs of the first subdomain (dd_load_adaptive_constraints)
    vector<double> cur = ci.matrix.empty() ? default_rows(A, ci) : ci.matrix;
    const int ncur = ci.used ? ci.ncdof : 0;
    const int ncol = ncur + nad;
    vector<double> mcol((size_t)nv * ncol, 0.0);
    for (int r = 0; r < ncur; ++r)
      for (int v = 0; v < nv; ++v) mcol[(size_t)r * nv + v] = cur[(size_t)r * nv + v];
    for (int r = 0; r < nad; ++r)
      for (int v = 0; v < nv; ++v) mcol[(size_t)(ncur + r) * nv + v] = cons[off + (size_t)r * P.n[p] + ci.idofi[v]];
    off += (long long)nad * P.n[p];
    int nvalid = 0;
    vector<double> qm = orthonormal_rows(nv, ncol, mcol, nvalid);
    // the second subdomain's face dofs in the first's order, by global dof
    std::unordered_map<int, int> gpos;
    for (int v = 0; v < nv; ++v) gpos.emplace(B.isvgvn[B.iivsvn[cj.idofi[v]]], v);
    ci.matrix.assign((size_t)nvalid * nv, 0.0);
    cj.matrix.assign((size_t)nvalid * nv, 0.0);
    for (int r = 0; r < nvalid; ++r)
      for (int v = 0; v < nv; ++v) {
        const double val = qm[(size_t)r * nv + v];
        ci.matrix[(size_t)r * nv + v] = val;
        auto it = gpos.find(A.isvgvn[A.iivsvn[ci.idofi[v]]]);
        if (it == gpos.end()) throw Error{ERR_NUMERIC, "face dof missing in the neighbouring subdomain"};
        cj.matrix[(size_t)r * nv + it->second] = val;
      }
    ci.ncdof = cj.ncdof = nvalid;
    ci.used = cj.used = nvalid > 0;
  }
  S.stats.nadaptive = nadaptive;
  host_constraint_rows(S);
}

}  // namespace bddc
