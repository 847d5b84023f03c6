// BDDC oracle: CPU restatement of the reference BDDC interface-PCG path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library in
// bddcml_gb300/: only tests/, __graft_entry__.smoke() and bench.py's
// cpu_baseline / reference legs may load it.  The product never links it.
//
// Parity status: unpinned against the reference's own outputs.  The reference
// (Fortran 95 + MPI + MUMPS + METIS + LAPACK) cannot be compiled here and ships
// no golden solver numbers; this restatement is pinned instead against direct
// sparse solves of the assembled global system (tests/test_oracle.py) and
// against structural invariants of the coarse space.
//
// What it restates (file:line in the reference project):
//   upload + matrix assembly ....... module_levels.f90:615-782, module_sm.f90:630-684
//   neighbours / interface ......... module_dd.f90:8071-8648 (dd_create_neighbouring),
//                                    module_utils.f90:878-945 (sorted intersection)
//   globs, corners, BC removal ..... module_dd.f90:8925-10016 (dd_create_globs),
//                                    10017-10327 (select_corners), 10329-10555 (coarse numbering)
//   BC elimination ................. module_dd.f90:1081-1256, module_sm.f90:431-600
//   interior factor (A11) .......... module_dd.f90:3983-4295 (blocking + factorisation)
//   weights ........................ module_dd.f90:11554-11722, 11800-11878
//   arithmetic constraints, C ...... module_dd.f90:4298-4384, 4869-5144, 11011-11235
//   augmented factor, coarse basis . module_dd.f90:5211-5799
//   reduced rhs, interior resolve .. module_dd.f90:6995-7257, 6811-6932
//   Schur apply .................... module_dd.f90:6564-6699
//   exchange (upload/download) ..... module_dd.f90:11236-11551
//   BDDC apply ..................... module_levels.f90:3627-4346
//   PCG + Lanczos estimate ......... module_krylov.f90:48-945, 2061-2118
//   BiCGSTAB, steepest descent ..... module_krylov.f90:948-1505, 1508-1840
//   coarse problem ................. module_levels.f90:3001-3170, 4029-4061
//
// The direct solver MUMPS is replaced by band Cholesky factorisations in the
// subdomain's own dof order.  The saddle-point system [A C^T; C 0] that the
// reference factors with a symmetric indefinite MUMPS (SYM=2) is solved here by
// an equivalent exact formulation: with A_r = A + sum_corner_dofs d_k e_k e_k^T
// (SPD once the corner constraints remove the kernel of A, and still banded),
// z = A_r^{-1}(f - C^T mu), mu = (C A_r^{-1} C^T)^{-1} C A_r^{-1} f.  On the
// constraint set C z = 0, A_r z = A z, so the solution is that of the
// reference system.  The coarse matrix is Phi^T A Phi, which equals the
// reference's -lambda (module_dd.f90:5615-5625) in exact arithmetic.
#include <algorithm>
#include <array>
#include <climits>
#include <cstdint>
#include <functional>
#include <unordered_map>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using std::vector;

namespace {

struct Band {
  // lower band Cholesky factor: L(i,j) for i-b <= j <= i stored at v[i*(b+1) + (j-i+b)]
  int n = 0, b = 0;
  vector<double> v;
  double& at(int i, int j) { return v[(size_t)i * (b + 1) + (j - i + b)]; }
  double at(int i, int j) const { return v[(size_t)i * (b + 1) + (j - i + b)]; }
  void factor() {
    for (int i = 0; i < n; ++i) {
      int j0 = std::max(0, i - b);
      for (int j = j0; j <= i; ++j) {
        double s = at(i, j);
        int k0 = std::max(j0, j - b);
        const double* li = &v[(size_t)i * (b + 1) + (k0 - i + b)];
        const double* lj = &v[(size_t)j * (b + 1) + (k0 - j + b)];
        for (int k = 0; k < j - k0; ++k) s -= li[k] * lj[k];
        if (i == j) {
          if (!(s > 0.0)) throw std::runtime_error("band Cholesky: non-positive pivot");
          at(i, i) = std::sqrt(s);
        } else {
          at(i, j) = s / at(j, j);
        }
      }
    }
  }
  void solve(double* x) const {  // L L^T x = rhs, in place
    for (int i = 0; i < n; ++i) {
      double s = x[i];
      int j0 = std::max(0, i - b);
      for (int j = j0; j < i; ++j) s -= at(i, j) * x[j];
      x[i] = s / at(i, i);
    }
    for (int i = n - 1; i >= 0; --i) {
      x[i] /= at(i, i);
      double xi = x[i];
      int j0 = std::max(0, i - b);
      for (int j = j0; j < i; ++j) x[j] -= at(i, j) * xi;
    }
  }
};

// dense symmetric positive definite (small): Cholesky in place, row-major n x n
static void dense_chol(vector<double>& a, int n, int nthreads = 1) {
  for (int j = 0; j < n; ++j) {
    double s = a[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) s -= a[(size_t)j * n + k] * a[(size_t)j * n + k];
    if (!(s > 0.0)) throw std::runtime_error("dense Cholesky: non-positive pivot");
    double d = std::sqrt(s);
    a[(size_t)j * n + j] = d;
#pragma omp parallel for schedule(static) num_threads(nthreads) if (n - j > 256 && nthreads > 1)
    for (int i = j + 1; i < n; ++i) {
      double t = a[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) t -= a[(size_t)i * n + k] * a[(size_t)j * n + k];
      a[(size_t)i * n + j] = t / d;
    }
  }
}
static void dense_chol_solve(const vector<double>& l, int n, double* x) {
  for (int i = 0; i < n; ++i) {
    double s = x[i];
    for (int k = 0; k < i; ++k) s -= l[(size_t)i * n + k] * x[k];
    x[i] = s / l[(size_t)i * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = x[i];
    for (int k = i + 1; k < n; ++k) s -= l[(size_t)k * n + i] * x[k];
    x[i] = s / l[(size_t)i * n + i];
  }
}

// General band matrix (nonsymmetric, matrixtype 0): A(i,j) for |i-j| <= b at
// v[i*(2b+1) + (j-i+b)], LU without pivoting in place (unit lower L, upper U).
// MUMPS factors the reference's general subdomain matrices with pivoting
// (module_mumps.f90:443-511); the test problems (convection-diffusion with cell
// Peclet numbers below 1) are diagonally dominant, where no pivot is needed.
struct BandLU {
  int n = 0, b = 0;
  vector<double> v;
  double& at(int i, int j) { return v[(size_t)i * (2 * b + 1) + (j - i + b)]; }
  double at(int i, int j) const { return v[(size_t)i * (2 * b + 1) + (j - i + b)]; }
  void factor() {
    for (int k = 0; k < n; ++k) {
      const double piv = at(k, k);
      if (!(std::fabs(piv) > 0.0)) throw std::runtime_error("band LU: zero pivot");
      for (int i = k + 1; i <= std::min(n - 1, k + b); ++i) {
        const double l = at(i, k) / piv;
        at(i, k) = l;
        if (l == 0.0) continue;
        for (int j = k + 1; j <= std::min(n - 1, k + b); ++j) at(i, j) -= l * at(k, j);
      }
    }
  }
  void solve(double* x) const {  // L U x = rhs, in place
    for (int i = 0; i < n; ++i) {
      double t = x[i];
      for (int j = std::max(0, i - b); j < i; ++j) t -= at(i, j) * x[j];
      x[i] = t;
    }
    for (int i = n - 1; i >= 0; --i) {
      double t = x[i];
      for (int j = i + 1; j <= std::min(n - 1, i + b); ++j) t -= at(i, j) * x[j];
      x[i] = t / at(i, i);
    }
  }
  void solve_t(double* x) const {  // (L U)^T x = rhs: U^T then L^T, in place
    for (int i = 0; i < n; ++i) {
      double t = x[i];
      for (int j = std::max(0, i - b); j < i; ++j) t -= at(j, i) * x[j];
      x[i] = t / at(i, i);
    }
    for (int i = n - 1; i >= 0; --i) {
      double t = x[i];
      for (int j = i + 1; j <= std::min(n - 1, i + b); ++j) t -= at(j, i) * x[j];
      x[i] = t;
    }
  }
};

// dense LU with partial pivoting (small general matrices: G = C A^-1 C^T and the
// coarse matrix of a nonsymmetric problem), row-major n x n, in place
static void dense_lu(vector<double>& a, int n, vector<int>& piv) {
  piv.resize(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(a[(size_t)i * n + k]) > std::fabs(a[(size_t)p * n + k])) p = i;
    piv[k] = p;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(a[(size_t)k * n + j], a[(size_t)p * n + j]);
    const double d = a[(size_t)k * n + k];
    if (!(std::fabs(d) > 0.0)) throw std::runtime_error("dense LU: singular matrix");
    for (int i = k + 1; i < n; ++i) {
      const double l = a[(size_t)i * n + k] / d;
      a[(size_t)i * n + k] = l;
      for (int j = k + 1; j < n; ++j) a[(size_t)i * n + j] -= l * a[(size_t)k * n + j];
    }
  }
}
// x <- A^-1 x (trans = false) or A^-T x (trans = true) with the factors of dense_lu
static void dense_lu_solve(const vector<double>& a, int n, const vector<int>& piv, double* x, bool trans) {
  if (!trans) {
    for (int k = 0; k < n; ++k) std::swap(x[k], x[piv[k]]);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < i; ++j) x[i] -= a[(size_t)i * n + j] * x[j];
    for (int i = n - 1; i >= 0; --i) {
      for (int j = i + 1; j < n; ++j) x[i] -= a[(size_t)i * n + j] * x[j];
      x[i] /= a[(size_t)i * n + i];
    }
  } else {
    for (int i = 0; i < n; ++i) {
      for (int j = 0; j < i; ++j) x[i] -= a[(size_t)j * n + i] * x[j];
      x[i] /= a[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; --i)
      for (int j = i + 1; j < n; ++j) x[i] -= a[(size_t)j * n + i] * x[j];
    for (int k = n - 1; k >= 0; --k) std::swap(x[k], x[piv[k]]);
  }
}

// COO sort + merge of duplicates (module_sm.f90:630-684 sm_assembly)
static void coo_assemble(vector<int>& ia, vector<int>& ja, vector<double>& a) {
  size_t n = ia.size();
  vector<size_t> p(n);
  std::iota(p.begin(), p.end(), 0);
  std::stable_sort(p.begin(), p.end(), [&](size_t x, size_t y) {
    return ia[x] != ia[y] ? ia[x] < ia[y] : ja[x] < ja[y];
  });
  vector<int> ni, nj;
  vector<double> na;
  ni.reserve(n); nj.reserve(n); na.reserve(n);
  for (size_t k = 0; k < n; ++k) {
    size_t q = p[k];
    if (!ni.empty() && ni.back() == ia[q] && nj.back() == ja[q]) na.back() += a[q];
    else { ni.push_back(ia[q]); nj.push_back(ja[q]); na.push_back(a[q]); }
  }
  ia.swap(ni); ja.swap(nj); a.swap(na);
}

static int find_index(const vector<int>& v, int x) {  // first position, -1 if absent
  for (size_t i = 0; i < v.size(); ++i) if (v[i] == x) return (int)i;
  return -1;
}

struct Cnode {
  int itype = 0;            // 3 corner, 2 edge, 1 face
  int global_cnode = 0;     // 1-based global coarse node number
  vector<int> insin;        // interface node indices
  vector<int> ivsivn;       // interface dof indices
  int nvar = 0;
  int ncdof = 0;            // constraints loaded
  vector<double> matrix;    // ncdof x nvar row-major
  bool used = false;
  vector<int> igcdof;       // global coarse dofs (1-based)
};

struct Sub {
  int isub = 0;  // 1-based
  int nelem = 0, nnod = 0, ndof = 0, ndim = 0;
  vector<int> inet, nnet, nndf, isngn, isvgvn, isegn, ifix;
  vector<double> xyz;  // xyz[d*nnod + i]
  vector<double> fixv, rhs, sol;
  bool rhs_complete = true;
  int matrixtype = 1;
  vector<int> ia, ja;  // 0-based, upper triangle
  vector<double> a;
  bool bc_present = false;
  vector<int> comp;  // nodal components (1-based)
  // neighbours / interface
  vector<int> iadj, nshnadj, ishnadj, ishnncadj;
  vector<int> iin, iivsvn, iovsvn;
  int nnodi = 0, ndofi = 0, ndofo = 0;
  vector<int> kdof;  // first dof of each node
  vector<int> kdofi; // first interface dof of each interface node (size nnodi+1)
  vector<int> xch_mine, xch_theirs, xch_ptr;  // exchange lists per neighbour (interface dof positions)
  // coarse space
  vector<int> icnsin;  // interface node index of corners (sorted by global id)
  vector<int> global_corner_number;
  vector<Cnode> cnodes;
  int nconstr = 0;
  vector<int> crow_ptr, crow_col;  // C in CSR over interface dofs
  vector<double> crow_val;
  vector<int> indrowc;             // global coarse dof of each row (1-based)
  // weights
  vector<double> wi;
  // BC
  vector<double> bc;
  // factors
  Band a11;                 // interior block in iovsvn order
  vector<int> c11_ptr, c11_col; vector<double> c11_val;  // full symmetric CSR of interior block (for checks)
  vector<int> a12_ptr, a12_col; vector<double> a12_val;  // CSR rows = interior, cols = interface
  vector<int> a22_ptr, a22_col; vector<double> a22_val;  // full symmetric CSR on interface
  Band aug;                 // A + corner shifts, full subdomain order
  // matrixtype 0 (general): LU factors in place of the Cholesky factors, the
  // interface-row block A_io, the dual basis from the adjoint problem
  // (module_dd.f90:5687-5757) and the LU pivots of G
  BandLU a11lu, auglu;
  vector<int> a21_ptr, a21_col; vector<double> a21_val;  // CSR rows = interface, cols = interior
  vector<double> ydual;     // ndof x nconstr: A_r^-T C^T
  vector<double> phisi_dual;
  vector<int> gpiv;
  vector<double> yaug;      // ndof x nconstr (column-major: yaug[c*ndof + i])
  vector<double> gchol;     // nconstr x nconstr Cholesky of C A_r^-1 C^T
  vector<double> phisi;     // ndofi x nconstr (column-major)
  vector<double> coarsem;   // nconstr x nconstr dense Phi^T A Phi
  vector<double> g, solo;
  // full symmetric CSR of the whole (BC-eliminated) matrix
  vector<int> f_ptr, f_col; vector<double> f_val;
  // fixed-rows matrix (upper triangle entries in a fixed row or column, before elimination)
  vector<int> fx_i, fx_j; vector<double> fx_v;
};

struct Oracle {
  int nsub = 0;
  int nthreads = 1;
  vector<Sub> subs;
  bool setup_done = false;
  int ncorner = 0, nedge = 0, nface = 0, ndofc = 0;
  vector<double> coarse_chol;  // dense Cholesky of the coarse matrix (LU for matrixtype 0)
  vector<int> coarse_piv;
  vector<int> ncdof_of_cnode;  // nndfc
  // adaptive face constraints (module_adaptivity.f90)
  bool adaptive = false;
  double adaptive_tau = 1.5;           // threshold_eigval_default, module_adaptivity.f90:30
  vector<std::array<int, 3>> pairs;    // (face global cnode, isub, jsub), 0-based subdomains
  vector<vector<double>> pair_eigs;    // largest eigenvalues per pair, descending
  vector<int> pair_nadaptive;          // eigenvalues >= tau per pair
  vector<int> face_ncdof;              // constraints per pair face after orthogonalisation
  double adaptivity_est = -1.0;
  // three levels: the level-2 problem built from this level's coarse space
  int nlevels = 2, nsub2 = 1;
  int setup_corner = 1, setup_arith = 1, setup_weights = 0;
  struct Oracle* lev2 = nullptr;
  ~Oracle();
  // Krylov recycling (module_krylov.f90:33-43): S-orthonormal search directions V and W = S V
  vector<vector<vector<double>>> rcv, rcw;  // [basis vector][subdomain][interface dof]
  int rc_cap = 0;
  std::string err;
  // PCG results
  vector<double> relres_hist;
};

// ---------------------------------------------------------------- helpers
static void sym_csr_from_upper(int n, const vector<int>& ia, const vector<int>& ja, const vector<double>& a,
                               vector<int>& ptr, vector<int>& col, vector<double>& val) {
  vector<int> cnt(n + 1, 0);
  for (size_t k = 0; k < ia.size(); ++k) {
    cnt[ia[k] + 1]++;
    if (ia[k] != ja[k]) cnt[ja[k] + 1]++;
  }
  for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  ptr = cnt;
  col.assign(ptr[n], 0);
  val.assign(ptr[n], 0.0);
  vector<int> pos(ptr.begin(), ptr.end() - 1);
  for (size_t k = 0; k < ia.size(); ++k) {
    col[pos[ia[k]]] = ja[k]; val[pos[ia[k]]++] = a[k];
    if (ia[k] != ja[k]) { col[pos[ja[k]]] = ia[k]; val[pos[ja[k]]++] = a[k]; }
  }
}

static void csr_mult(const vector<int>& ptr, const vector<int>& col, const vector<double>& val,
                     const double* x, double* y, int nrow) {
  for (int i = 0; i < nrow; ++i) {
    double s = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) s += val[k] * x[col[k]];
    y[i] = s;
  }
}

// CSR rows of a general (matrixtype 0) COO matrix
static void csr_from_full(int n, const vector<int>& ia, const vector<int>& ja, const vector<double>& a,
                          vector<int>& ptr, vector<int>& col, vector<double>& val) {
  vector<int> cnt(n + 1, 0);
  for (size_t k = 0; k < ia.size(); ++k) cnt[ia[k] + 1]++;
  for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  ptr = cnt;
  col.assign(ptr[n], 0);
  val.assign(ptr[n], 0.0);
  vector<int> pos(ptr.begin(), ptr.end() - 1);
  for (size_t k = 0; k < ia.size(); ++k) { col[pos[ia[k]]] = ja[k]; val[pos[ia[k]]++] = a[k]; }
}

// nodal components from the dual mesh graph (module_dd.f90:2516-2770):
// elements sharing at least `neighbouring` nodes are connected.
static void nodal_components(Sub& s, bool find_components, int neighbouring) {
  s.comp.assign(s.nnod, 1);
  if (!find_components || s.nelem == 0) return;
  vector<int> kinet(s.nelem + 1, 0);
  for (int e = 0; e < s.nelem; ++e) kinet[e + 1] = kinet[e] + s.nnet[e];
  vector<vector<int>> node_elems(s.nnod);
  for (int e = 0; e < s.nelem; ++e)
    for (int k = kinet[e]; k < kinet[e + 1]; ++k) node_elems[s.inet[k]].push_back(e);
  vector<int> ecomp(s.nelem, 0);
  int ncomp = 0;
  vector<int> cntshared(s.nelem, 0), touched;
  for (int e0 = 0; e0 < s.nelem; ++e0) {
    if (ecomp[e0]) continue;
    ++ncomp;
    vector<int> stack{e0};
    ecomp[e0] = ncomp;
    while (!stack.empty()) {
      int e = stack.back(); stack.pop_back();
      touched.clear();
      for (int k = kinet[e]; k < kinet[e + 1]; ++k)
        for (int f : node_elems[s.inet[k]]) {
          if (f == e) continue;
          if (cntshared[f]++ == 0) touched.push_back(f);
        }
      for (int f : touched) {
        if (cntshared[f] >= neighbouring && !ecomp[f]) { ecomp[f] = ncomp; stack.push_back(f); }
        cntshared[f] = 0;
      }
    }
  }
  for (int e = 0; e < s.nelem; ++e)
    for (int k = kinet[e]; k < kinet[e + 1]; ++k) s.comp[s.inet[k]] = ecomp[e];
}

static vector<int> sorted_intersection(vector<int> a, vector<int> b) {
  std::sort(a.begin(), a.end());
  std::sort(b.begin(), b.end());
  vector<int> out;
  std::set_intersection(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(out));
  return out;
}

}  // namespace

// ============================================================ neighbours
static void create_neighbouring(Oracle& o) {
  int nsub = o.nsub;
  // guess by node-id ranges and coordinate bounding boxes (module_dd.f90:8649-8924);
  // the guess only has to be a superset, the intersection decides.
  vector<int> lo(nsub), hi(nsub);
  vector<double> bmin(3 * nsub), bmax(3 * nsub);
  for (int s = 0; s < nsub; ++s) {
    auto& S = o.subs[s];
    lo[s] = *std::min_element(S.isngn.begin(), S.isngn.end());
    hi[s] = *std::max_element(S.isngn.begin(), S.isngn.end());
    for (int d = 0; d < S.ndim; ++d) {
      const double* x = &S.xyz[(size_t)d * S.nnod];
      bmin[3 * s + d] = *std::min_element(x, x + S.nnod);
      bmax[3 * s + d] = *std::max_element(x, x + S.nnod);
    }
  }
  vector<vector<int>> sorted_ids(nsub);
  for (int s = 0; s < nsub; ++s) { sorted_ids[s] = o.subs[s].isngn; std::sort(sorted_ids[s].begin(), sorted_ids[s].end()); }
#pragma omp parallel for schedule(dynamic) num_threads(o.nthreads)
  for (int s = 0; s < nsub; ++s) {
    auto& S = o.subs[s];
    std::map<int, int> gid2loc;
    for (int i = 0; i < S.nnod; ++i) gid2loc.emplace(S.isngn[i], i);
    vector<int> kinodes(S.nnod, 0);
    vector<vector<int>> shared_g;  // per actual neighbour, sorted global ids
    vector<int> adj;
    for (int t = 0; t < nsub; ++t) {
      if (t == s) continue;
      if (lo[s] > hi[t] || hi[s] < lo[t]) continue;
      bool bb = true;
      for (int d = 0; d < S.ndim; ++d) {
        double tol = 1e-9 * (1.0 + std::fabs(bmax[3 * s + d]) + std::fabs(bmax[3 * t + d]));
        if (bmin[3 * s + d] > bmax[3 * t + d] + tol || bmax[3 * s + d] < bmin[3 * t + d] - tol) bb = false;
      }
      if (!bb) continue;
      vector<int> inter;
      std::set_intersection(sorted_ids[s].begin(), sorted_ids[s].end(), sorted_ids[t].begin(), sorted_ids[t].end(),
                            std::back_inserter(inter));
      if (inter.empty()) continue;
      adj.push_back(t + 1);
      for (int g : inter) kinodes[gid2loc[g]]++;
      shared_g.push_back(std::move(inter));
    }
    // interface: nodes shared with anybody, in local order (module_dd.f90:8410-8470)
    S.kdof.assign(S.nnod, 0);
    for (int i = 1; i < S.nnod; ++i) S.kdof[i] = S.kdof[i - 1] + S.nndf[i - 1];
    S.iin.clear(); S.iivsvn.clear(); S.iovsvn.clear();
    vector<int> inodi_of(S.nnod, -1);
    for (int i = 0; i < S.nnod; ++i) {
      if (kinodes[i] > 0) {
        inodi_of[i] = (int)S.iin.size();
        S.iin.push_back(i);
        for (int d = 0; d < S.nndf[i]; ++d) S.iivsvn.push_back(S.kdof[i] + d);
      } else {
        for (int d = 0; d < S.nndf[i]; ++d) S.iovsvn.push_back(S.kdof[i] + d);
      }
    }
    S.nnodi = (int)S.iin.size();
    S.ndofi = (int)S.iivsvn.size();
    S.ndofo = (int)S.iovsvn.size();
    S.iadj = adj;
    S.nshnadj.clear(); S.ishnadj.clear(); S.ishnncadj.clear();
    for (size_t a = 0; a < adj.size(); ++a) {
      auto& T = o.subs[adj[a] - 1];
      S.nshnadj.push_back((int)shared_g[a].size());
      std::unordered_map<int, int> tloc;
      for (int i = 0; i < T.nnod; ++i) tloc.emplace(T.isngn[i], i);
      for (int g : shared_g[a]) {
        S.ishnadj.push_back(inodi_of[gid2loc[g]]);
        S.ishnncadj.push_back(T.comp[tloc.at(g)]);
      }
    }
  }
}

// ================================================================ globs
static void create_globs(Oracle& o, bool use_corner_constraints, int meshdim) {
  int nsub = o.nsub;
  struct Aux {
    vector<int> nsubnode;                // per interface node
    vector<vector<std::array<int, 3>>> globsubs;
    vector<int> globtypes, kglobs;
    vector<int> icgn;                    // corners by global node id
    int ncorners = 0, nedges = 0, nfaces = 0;
    vector<int> iegn, ifgn;
    vector<int> icgcn, iegcn, ifgcn;
    vector<int> iingns;
  };
  vector<Aux> aux(nsub);
  // ---- pass 1: classification + corner selection (module_dd.f90:9099-9276, 10017-10327)
  for (int s = 0; s < nsub; ++s) {
    auto& S = o.subs[s];
    auto& A = aux[s];
    int nnodi = S.nnodi;
    A.nsubnode.assign(nnodi, 0);
    A.globsubs.assign(nnodi, {});
    int k = 0;
    for (size_t ia = 0; ia < S.iadj.size(); ++ia) {
      for (int ish = 0; ish < S.nshnadj[ia]; ++ish) {
        int inodi = S.ishnadj[k + ish];
        int mycomp = S.comp[S.iin[inodi]];
        A.nsubnode[inodi]++;
        A.globsubs[inodi].push_back({S.iadj[ia], S.ishnncadj[k + ish], mycomp});
      }
      k += S.nshnadj[ia];
    }
    for (int i = 0; i < nnodi; ++i)
      if (A.nsubnode[i] == 0) throw std::runtime_error("interface coverage by globs failed");
    A.globtypes.assign(nnodi, 0);
    A.kglobs.assign(nnodi, -1);
    int iglobs = 0;
    for (int i = 0; i < nnodi; ++i) {
      if (A.kglobs[i] != -1) continue;
      ++iglobs;
      A.kglobs[i] = iglobs;
      int nsubn = A.nsubnode[i];
      int nglobn = 1;
      for (int j = i + 1; j < nnodi; ++j) {
        if (A.kglobs[j] == -1 && A.globtypes[j] != 3 && A.nsubnode[j] == nsubn && A.globsubs[j] == A.globsubs[i]) {
          A.kglobs[j] = iglobs;
          nglobn++;
          A.globtypes[j] = (nsubn == 1) ? 1 : 2;
        }
      }
      if (nsubn == 1) A.globtypes[i] = 1;
      else A.globtypes[i] = (nglobn > 1) ? 2 : 3;
    }
    for (int i = 0; i < nnodi; ++i) if (A.nsubnode[i] == 1) A.globtypes[i] = 1;
    if (use_corner_constraints) {
      int kk = 0;
      for (size_t ia = 0; ia < S.iadj.size(); ++ia) {
        int nshn = S.nshnadj[ia];
        bool face = false;
        for (int ish = 0; ish < nshn; ++ish)
          if (A.globtypes[S.ishnadj[kk + ish]] == 1) { face = true; break; }
        if (face) {
          // interface components (check_face_components = .true.)
          vector<int> myc(nshn), adjc(nshn);
          for (int ish = 0; ish < nshn; ++ish) {
            myc[ish] = S.comp[S.iin[S.ishnadj[kk + ish]]];
            adjc[ish] = S.ishnncadj[kk + ish];
          }
          auto compress = [](vector<int>& v) {
            int mx = *std::max_element(v.begin(), v.end());
            int nw = 0;
            for (int old = 1; old <= mx; ++old) {
              if (std::find(v.begin(), v.end(), old) != v.end()) {
                ++nw;
                for (auto& x : v) if (x == old) x = nw;
              }
            }
            return nw;
          };
          compress(myc);
          int nadjc = compress(adjc);
          vector<int> ic(nshn);
          for (int ish = 0; ish < nshn; ++ish) ic[ish] = (myc[ish] - 1) * nadjc + adjc[ish];
          int nic = compress(ic);
          for (int icomp = 1; icomp <= nic; ++icomp) {
            vector<int> compind;
            for (int ish = 0; ish < nshn; ++ish) if (ic[ish] == icomp) compind.push_back(ish);
            int m = (int)compind.size();
            int ndim = S.ndim;
            vector<double> xs(m * 3, 0.0);
            for (int c = 0; c < m; ++c) {
              int nd = S.iin[S.ishnadj[kk + compind[c]]];
              for (int d = 0; d < ndim; ++d) xs[c * 3 + d] = S.xyz[(size_t)d * S.nnod + nd];
            }
            int inodcf[4] = {0, 0, 0, 0};  // 1-based positions, 0 = none
            auto farthest_from = [&](int base) {
              double best = -1.0; int loc = 0;
              for (int c = 0; c < m; ++c) {
                double dist = 0.0;
                for (int d = 0; d < ndim; ++d) { double t = xs[c * 3 + d] - xs[base * 3 + d]; dist += t * t; }
                if (dist > best) { best = dist; loc = c; }  // maxloc: first maximum
              }
              return loc + 1;
            };
            if (m > 0) inodcf[0] = farthest_from(0);
            if (meshdim > 1 && m > 1) {
              inodcf[1] = farthest_from(inodcf[0] - 1);
              if (inodcf[1] == inodcf[0]) {
                for (int c = 1; c <= m; ++c) if (c != inodcf[0]) { inodcf[1] = c; break; }
              }
            }
            if (meshdim > 2 && m > 2) {
              double x1 = xs[(inodcf[0] - 1) * 3], y1 = xs[(inodcf[0] - 1) * 3 + 1], z1 = xs[(inodcf[0] - 1) * 3 + 2];
              double x2 = xs[(inodcf[1] - 1) * 3], y2 = xs[(inodcf[1] - 1) * 3 + 1], z2 = xs[(inodcf[1] - 1) * 3 + 2];
              vector<double> area(m);
              for (int c = 0; c < m; ++c) {
                double xi = xs[c * 3], yi = xs[c * 3 + 1], zi = xs[c * 3 + 2];
                double t1 = (y2 - y1) * (zi - z1) - (yi - y1) * (z2 - z1);
                double t2 = (x2 - x1) * (zi - z1) - (xi - x1) * (z2 - z1);
                double t3 = (x2 - x1) * (yi - y1) - (xi - x1) * (y2 - y1);
                area[c] = t1 * t1 + t2 * t2 + t3 * t3;
              }
              for (int round = 1; round <= 2; ++round) {
                double maxv = 0.0; int maxl = 0;
                if (round == 1) { for (int c = 0; c < m; ++c) if (area[c] > maxv) { maxv = area[c]; maxl = c + 1; } }
                else { for (int c = m - 1; c >= 0; --c) if (area[c] > maxv) { maxv = area[c]; maxl = c + 1; } }
                inodcf[1 + round] = maxl;
              }
              if ((inodcf[2] == inodcf[0] && inodcf[3] == inodcf[0]) || (inodcf[2] == inodcf[1] && inodcf[3] == inodcf[1])) {
                for (int c = 1; c <= m; ++c) if (c != inodcf[0] && c != inodcf[1]) { inodcf[2] = c; break; }
                for (int c = 1; c <= m; ++c) if (c != inodcf[0] && c != inodcf[1] && c != inodcf[2]) { inodcf[3] = c; break; }
              }
            }
            int end_bound = meshdim <= 2 ? 2 : 4;
            for (int i = 0; i < end_bound; ++i)
              if (inodcf[i] != 0) A.globtypes[S.ishnadj[kk + compind[inodcf[i] - 1]]] = 3;
          }
        }
        kk += nshn;
      }
    }
    A.icgn.clear();
    for (int i = 0; i < nnodi; ++i) if (A.globtypes[i] == 3) A.icgn.push_back(S.isngn[S.iin[i]]);
    A.iingns.resize(nnodi);
    for (int i = 0; i < nnodi; ++i) A.iingns[i] = S.isngn[S.iin[i]];
  }
  // ---- corner merge across neighbours (module_dd.f90:9296-9385)
  vector<vector<int>> newicgn(nsub);
  for (int s = 0; s < nsub; ++s) {
    auto& S = o.subs[s];
    vector<int> merge = aux[s].icgn;
    for (int t : S.iadj) merge.insert(merge.end(), aux[t - 1].icgn.begin(), aux[t - 1].icgn.end());
    std::sort(merge.begin(), merge.end());
    merge.erase(std::unique(merge.begin(), merge.end()), merge.end());
    newicgn[s] = sorted_intersection(aux[s].iingns, merge);
  }
  for (int s = 0; s < nsub; ++s) {
    aux[s].icgn = newicgn[s];
    aux[s].ncorners = (int)aux[s].icgn.size();
    for (int g : aux[s].icgn) aux[s].globtypes[find_index(aux[s].iingns, g)] = 3;
  }
  // ---- coarse numbering of a class of entities (module_dd.f90:10329-10555)
  auto number = [&](int shift, std::function<vector<int>&(Aux&)> gidx, std::function<vector<int>&(Aux&)> gcidx) {
    vector<int> nuniq(nsub + 1, 0);
    for (int s = 0; s < nsub; ++s) {
      auto& A = aux[s];
      int isub = s + 1, cnt = 0;
      for (int g : gidx(A)) {
        int inodi = find_index(A.iingns, g);
        int mn = isub;
        for (auto& t : A.globsubs[inodi]) mn = std::min(mn, t[0]);
        if (mn == isub) cnt++;
      }
      nuniq[s] = cnt;
    }
    vector<int> start(nsub + 1);
    start[0] = 1;
    for (int s = 0; s < nsub; ++s) start[s + 1] = start[s] + nuniq[s];
    int ncoarse = start[nsub] - 1;
    std::map<int, int> owned;  // global entity id -> coarse number
    for (int s = 0; s < nsub; ++s) {
      auto& A = aux[s];
      auto& S = o.subs[s];
      auto& gi = gidx(A);
      auto& gc = gcidx(A);
      gc.assign(gi.size(), 0);
      int indcg = start[s];
      int isub = s + 1;
      for (int inodi = 0; inodi < S.nnodi; ++inodi) {
        int g = A.iingns[inodi];
        int pos = find_index(gi, g);
        if (pos < 0) continue;
        int mn = isub;
        for (auto& t : A.globsubs[inodi]) mn = std::min(mn, t[0]);
        if (mn == isub) { gc[pos] = shift + indcg; owned[g] = shift + indcg; indcg++; }
      }
    }
    for (int s = 0; s < nsub; ++s) {
      auto& gi = gidx(aux[s]);
      auto& gc = gcidx(aux[s]);
      for (size_t k = 0; k < gi.size(); ++k)
        if (gc[k] == 0) {
          auto it = owned.find(gi[k]);
          if (it == owned.end()) throw std::runtime_error("coarse entity without owner");
          gc[k] = it->second;
        }
    }
    return ncoarse;
  };
  o.ncorner = number(0, [](Aux& A) -> vector<int>& { return A.icgn; }, [](Aux& A) -> vector<int>& { return A.icgcn; });
  for (int s = 0; s < nsub; ++s) {
    auto& S = o.subs[s];
    auto& A = aux[s];
    S.icnsin.assign(A.ncorners, -1);
    for (int c = 0; c < A.ncorners; ++c) S.icnsin[c] = find_index(A.iingns, A.icgn[c]);
    S.global_corner_number = A.icgcn;
  }
  // ---- pass 2: edges, faces, BC removal (module_dd.f90:9387-9587)
  for (int s = 0; s < nsub; ++s) {
    auto& S = o.subs[s];
    auto& A = aux[s];
    int nnodi = S.nnodi;
    A.kglobs.assign(nnodi, -1);
    A.globtypes.assign(nnodi, 0);
    int nc = A.ncorners;
    for (int c = 0; c < nc; ++c) { A.kglobs[S.icnsin[c]] = c + 1; A.globtypes[S.icnsin[c]] = 3; }
    int iedges = 0;
    for (int i = 0; i < nnodi; ++i) {
      if (A.kglobs[i] != -1) continue;
      int nsubn = A.nsubnode[i];
      if (nsubn > 1) {
        ++iedges;
        A.kglobs[i] = nc + iedges; A.globtypes[i] = 2;
        for (int j = i + 1; j < nnodi; ++j)
          if (A.kglobs[j] == -1 && A.nsubnode[j] == nsubn && A.globsubs[j] == A.globsubs[i]) {
            A.kglobs[j] = nc + iedges; A.globtypes[j] = 2;
          }
      }
    }
    int nedges = iedges, ifaces = 0;
    for (int i = 0; i < nnodi; ++i) {
      if (A.kglobs[i] != -1) continue;
      int nsubn = A.nsubnode[i];
      if (nsubn != 1) throw std::runtime_error("unassigned non-face node");
      ++ifaces;
      A.kglobs[i] = nc + nedges + ifaces; A.globtypes[i] = 1;
      for (int j = i + 1; j < nnodi; ++j)
        if (A.kglobs[j] == -1 && A.nsubnode[j] == nsubn && A.globsubs[j] == A.globsubs[i]) {
          A.kglobs[j] = nc + nedges + ifaces; A.globtypes[j] = 1;
        }
    }
    int nfaces = ifaces;
    if (S.bc_present) {  // remove_bc_nodes on level 1
      for (int i = 0; i < nnodi; ++i) {
        if (A.globtypes[i] == 3) continue;
        int nd = S.iin[i];
        bool fixed = false;
        for (int d = 0; d < S.nndf[nd]; ++d) if (S.ifix[S.kdof[nd] + d] > 0) fixed = true;
        if (fixed) { A.kglobs[i] = -2; A.globtypes[i] = -2; }
      }
      int ie = 0;
      for (int e = 1; e <= nedges; ++e) {
        int old = nc + e;
        if (std::find(A.kglobs.begin(), A.kglobs.end(), old) != A.kglobs.end()) {
          ++ie;
          for (auto& x : A.kglobs) if (x == old) x = nc + ie;
        }
      }
      int iff = 0;
      for (int f = 1; f <= nfaces; ++f) {
        int old = nc + nedges + f;
        if (std::find(A.kglobs.begin(), A.kglobs.end(), old) != A.kglobs.end()) {
          ++iff;
          for (auto& x : A.kglobs) if (x == old) x = nc + ie + iff;
        }
      }
      nedges = ie; nfaces = iff;
    }
    A.nedges = nedges; A.nfaces = nfaces;
    A.iegn.assign(nedges, 0);
    A.ifgn.assign(nfaces, 0);
    for (int e = 0; e < nedges; ++e) {
      int mn = INT32_MAX;
      for (int i = 0; i < nnodi; ++i) if (A.kglobs[i] == nc + e + 1) mn = std::min(mn, A.iingns[i]);
      A.iegn[e] = mn;
    }
    for (int f = 0; f < nfaces; ++f) {
      int mn = INT32_MAX;
      for (int i = 0; i < nnodi; ++i) if (A.kglobs[i] == nc + nedges + f + 1) mn = std::min(mn, A.iingns[i]);
      A.ifgn[f] = mn;
    }
  }
  o.nedge = number(o.ncorner, [](Aux& A) -> vector<int>& { return A.iegn; }, [](Aux& A) -> vector<int>& { return A.iegcn; });
  o.nface = number(o.ncorner + o.nedge, [](Aux& A) -> vector<int>& { return A.ifgn; }, [](Aux& A) -> vector<int>& { return A.ifgcn; });
  // ---- cnodes (module_dd.f90:4869-5016)
  for (int s = 0; s < nsub; ++s) {
    auto& S = o.subs[s];
    auto& A = aux[s];
    vector<int> kdofi(S.nnodi, 0);
    for (int i = 1; i < S.nnodi; ++i) kdofi[i] = kdofi[i - 1] + S.nndf[S.iin[i - 1]];
    S.cnodes.clear();
    for (int c = 0; c < A.ncorners; ++c) {
      Cnode cn;
      cn.itype = 3;
      cn.global_cnode = S.global_corner_number[c];
      int in = S.icnsin[c];
      cn.insin = {in};
      cn.nvar = S.nndf[S.iin[in]];
      for (int d = 0; d < cn.nvar; ++d) cn.ivsivn.push_back(kdofi[in] + d);
      S.cnodes.push_back(cn);
    }
    int nc = A.ncorners;
    for (int gl = 0; gl < A.nedges + A.nfaces; ++gl) {
      Cnode cn;
      bool edge = gl < A.nedges;
      cn.itype = edge ? 2 : 1;
      cn.global_cnode = edge ? A.iegcn[gl] : A.ifgcn[gl - A.nedges];
      for (int i = 0; i < S.nnodi; ++i)
        if (A.kglobs[i] == nc + gl + 1) {
          cn.insin.push_back(i);
          for (int d = 0; d < S.nndf[S.iin[i]]; ++d) cn.ivsivn.push_back(kdofi[i] + d);
        }
      cn.nvar = (int)cn.ivsivn.size();
      S.cnodes.push_back(cn);
    }
  }
}

// arithmetic constraints of one glob type (module_dd.f90:4298-4384)
static void load_arithmetic_constraints(Sub& S, int itype) {
  for (auto& cn : S.cnodes) {
    if (cn.itype != itype) continue;
    int ncdof = 0;
    for (int in : cn.insin) ncdof = std::max(ncdof, S.nndf[S.iin[in]]);
    vector<double> m((size_t)ncdof * cn.nvar, 0.0);
    int p = 0;
    for (int in : cn.insin) {
      int nd = S.nndf[S.iin[in]];
      for (int d = 0; d < nd; ++d) m[(size_t)d * cn.nvar + p + d] = 1.0;
      p += nd;
    }
    cn.matrix.insert(cn.matrix.end(), m.begin(), m.end());
    cn.ncdof += ncdof;
    cn.used = true;
  }
}

// ================================================================ dense helpers for adaptivity
// Symmetric eigen-decomposition of a (n x n, row-major, overwritten): Householder
// reduction to tridiagonal form, then implicit QR steps with Wilkinson shifts
// (the textbook method of LAPACK's DSYEV/DSYGV, used by module_adaptivity.f90
// for dense eigenproblems).  Eigenvalues ascending in w; z(i, k) = z[i*n + k]
// holds the k-th eigenvector.
static void sym_eig(int n, vector<double>& a, vector<double>& w, vector<double>& z) {
  z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) z[(size_t)i * n + i] = 1.0;
  vector<double> v(n), p(n);
  for (int k = 0; k + 2 < n; ++k) {
    const int m = n - k - 1;  // size of the trailing block
    double nx = 0.0;
    for (int i = 0; i < m; ++i) nx += a[(size_t)(k + 1 + i) * n + k] * a[(size_t)(k + 1 + i) * n + k];
    nx = std::sqrt(nx);
    if (nx == 0.0) continue;
    const double x0 = a[(size_t)(k + 1) * n + k];
    const double alpha = x0 > 0 ? -nx : nx;
    for (int i = 0; i < m; ++i) v[i] = a[(size_t)(k + 1 + i) * n + k];
    v[0] -= alpha;
    double nv = 0.0;
    for (int i = 0; i < m; ++i) nv += v[i] * v[i];
    nv = std::sqrt(nv);
    if (nv == 0.0) continue;
    for (int i = 0; i < m; ++i) v[i] /= nv;
    // trailing block A <- H A H with H = I - 2 v v^T
    double kk = 0.0;
    for (int i = 0; i < m; ++i) {
      double t = 0.0;
      for (int j = 0; j < m; ++j) t += a[(size_t)(k + 1 + i) * n + k + 1 + j] * v[j];
      p[i] = t;
      kk += v[i] * t;
    }
    for (int i = 0; i < m; ++i) p[i] -= kk * v[i];
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < m; ++j) a[(size_t)(k + 1 + i) * n + k + 1 + j] -= 2.0 * (v[i] * p[j] + p[i] * v[j]);
    a[(size_t)(k + 1) * n + k] = a[(size_t)k * n + k + 1] = alpha;
    for (int i = 1; i < m; ++i) a[(size_t)(k + 1 + i) * n + k] = a[(size_t)k * n + k + 1 + i] = 0.0;
    // z <- z H on columns k+1 ..
    for (int r = 0; r < n; ++r) {
      double t = 0.0;
      for (int j = 0; j < m; ++j) t += z[(size_t)r * n + k + 1 + j] * v[j];
      for (int j = 0; j < m; ++j) z[(size_t)r * n + k + 1 + j] -= 2.0 * t * v[j];
    }
  }
  vector<double> d(n), e(std::max(1, n - 1), 0.0);
  for (int i = 0; i < n; ++i) d[i] = a[(size_t)i * n + i];
  for (int i = 0; i + 1 < n; ++i) e[i] = a[(size_t)i * n + i + 1];
  const double eps = 2.220446049250313e-16;
  int hi = n - 1, guard = 0;
  while (hi > 0) {
    if (std::fabs(e[hi - 1]) <= eps * (std::fabs(d[hi - 1]) + std::fabs(d[hi]))) { e[hi - 1] = 0.0; --hi; continue; }
    int lo = hi - 1;
    while (lo > 0 && std::fabs(e[lo - 1]) > eps * (std::fabs(d[lo - 1]) + std::fabs(d[lo]))) --lo;
    if (lo > 0) e[lo - 1] = 0.0;
    if (++guard > 60 * n) throw std::runtime_error("symmetric eigen-decomposition did not converge");
    // Wilkinson shift from the trailing 2x2 block
    const double dl = 0.5 * (d[hi - 1] - d[hi]);
    const double b = e[hi - 1];
    const double mu = d[hi] - b * b / (dl + (dl >= 0 ? 1.0 : -1.0) * std::hypot(dl, b));
    double x = d[lo] - mu, zz = e[lo];
    for (int k = lo; k < hi; ++k) {
      const double r = std::hypot(x, zz);
      const double c = r == 0.0 ? 1.0 : x / r, sn = r == 0.0 ? 0.0 : zz / r;
      if (k > lo) e[k - 1] = r;
      const double ak = d[k], ak1 = d[k + 1], bk = e[k];
      d[k] = c * c * ak + 2.0 * c * sn * bk + sn * sn * ak1;
      d[k + 1] = sn * sn * ak - 2.0 * c * sn * bk + c * c * ak1;
      e[k] = c * sn * (ak1 - ak) + (c * c - sn * sn) * bk;
      if (k + 1 < hi) {  // bulge below the block
        x = e[k];
        zz = sn * e[k + 1];
        e[k + 1] *= c;
      }
      for (int r2 = 0; r2 < n; ++r2) {
        const double zk = z[(size_t)r2 * n + k], zk1 = z[(size_t)r2 * n + k + 1];
        z[(size_t)r2 * n + k] = c * zk + sn * zk1;
        z[(size_t)r2 * n + k + 1] = -sn * zk + c * zk1;
      }
    }
  }
  // sort ascending
  vector<int> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::sort(ord.begin(), ord.end(), [&](int x1, int x2) { return d[x1] < d[x2]; });
  w.resize(n);
  vector<double> zs((size_t)n * n);
  for (int k = 0; k < n; ++k) {
    w[k] = d[ord[k]];
    for (int r2 = 0; r2 < n; ++r2) zs[(size_t)r2 * n + k] = z[(size_t)r2 * n + ord[k]];
  }
  z.swap(zs);
}

// Householder QR with column pivoting of the nrow x ncol matrix m (column-major,
// overwritten), then the first nvalid columns of Q, where nvalid counts the
// leading |R_ii| >= 0.01 |R_11| (dd_orthogonalize_constraints, module_dd.f90:4637-4760,
// DGEQP3 + DORGQR).  Returns Q (nrow x nvalid, column-major).
static vector<double> pivoted_orthonormal_basis(int nrow, int ncol, vector<double> m, int& nvalid) {
  const int kmax = std::min(nrow, ncol);
  vector<vector<double>> refl;
  vector<double> rdiag;
  vector<int> piv(ncol);
  std::iota(piv.begin(), piv.end(), 0);
  for (int k = 0; k < kmax; ++k) {
    int best = k;
    double bn = -1.0;
    for (int c = k; c < ncol; ++c) {
      double t = 0.0;
      for (int r = k; r < nrow; ++r) t += m[(size_t)c * nrow + r] * m[(size_t)c * nrow + r];
      if (t > bn) { bn = t; best = c; }
    }
    if (best != k) {
      for (int r = 0; r < nrow; ++r) std::swap(m[(size_t)k * nrow + r], m[(size_t)best * nrow + r]);
      std::swap(piv[k], piv[best]);
    }
    double nx = std::sqrt(std::max(0.0, bn));
    vector<double> v(nrow, 0.0);
    if (nx == 0.0) { rdiag.push_back(0.0); refl.push_back(v); continue; }
    const double x0 = m[(size_t)k * nrow + k];
    const double alpha = x0 > 0 ? -nx : nx;
    for (int r = k; r < nrow; ++r) v[r] = m[(size_t)k * nrow + r];
    v[k] -= alpha;
    double nv = 0.0;
    for (int r = k; r < nrow; ++r) nv += v[r] * v[r];
    nv = std::sqrt(nv);
    if (nv > 0) for (int r = k; r < nrow; ++r) v[r] /= nv;
    for (int c = k; c < ncol; ++c) {
      double t = 0.0;
      for (int r = k; r < nrow; ++r) t += v[r] * m[(size_t)c * nrow + r];
      for (int r = k; r < nrow; ++r) m[(size_t)c * nrow + r] -= 2.0 * t * v[r];
    }
    rdiag.push_back(m[(size_t)k * nrow + k]);
    refl.push_back(v);
  }
  nvalid = 0;
  if (kmax > 0 && std::fabs(rdiag[0]) > 1e-12) {
    const double th = 0.01 * std::fabs(rdiag[0]);
    for (int i = 0; i < kmax; ++i) {
      if (std::fabs(rdiag[i]) < th) break;
      nvalid = i + 1;
    }
  }
  vector<double> q((size_t)nrow * nvalid, 0.0);
  for (int c = 0; c < nvalid; ++c) {
    double* col = &q[(size_t)c * nrow];
    col[c] = 1.0;
    for (int k = nvalid - 1; k >= 0; --k) {
      const auto& v = refl[k];
      double t = 0.0;
      for (int r = k; r < nrow; ++r) t += v[r] * col[r];
      for (int r = k; r < nrow; ++r) col[r] -= 2.0 * t * v[r];
    }
  }
  return q;
}

// ================================================================ API
extern "C" {

void* oracle_create(int nsub, int nthreads) {
  auto* o = new Oracle;
  o->nsub = nsub;
  o->nthreads = std::max(1, nthreads);
  o->subs.resize(nsub);
  return o;
}

void oracle_destroy(void* h) { delete static_cast<Oracle*>(h); }

const char* oracle_error(void* h) { return static_cast<Oracle*>(h)->err.c_str(); }

// All index arrays 0-based.  xyz is (nnod x ndim) column-major as in the ABI.
int oracle_upload(void* h, int isub, int nelem, int nnod, int ndof, int ndim,
                  const int* inet, int linet, const int* nnet, const int* nndf,
                  const int* isngn, const int* isvgvn, const int* isegn, const double* xyz,
                  const int* ifix, const double* fixv, const double* rhs, int is_rhs_complete,
                  const double* sol, int matrixtype, int la, const int* i_sparse, const int* j_sparse,
                  const double* a_sparse, int find_components, int neighbouring) {
  auto* o = static_cast<Oracle*>(h);
  if (isub < 0 || isub >= o->nsub) { o->err = "bad isub"; return 1; }
  Sub& S = o->subs[isub];
  S.isub = isub + 1;
  S.nelem = nelem; S.nnod = nnod; S.ndof = ndof; S.ndim = ndim;
  S.inet.assign(inet, inet + linet);
  S.nnet.assign(nnet, nnet + nelem);
  S.nndf.assign(nndf, nndf + nnod);
  S.isngn.assign(isngn, isngn + nnod);
  S.isvgvn.assign(isvgvn, isvgvn + ndof);
  S.isegn.assign(isegn, isegn + nelem);
  S.xyz.assign(xyz, xyz + (size_t)nnod * ndim);
  S.ifix.assign(ifix, ifix + ndof);
  S.fixv.assign(fixv, fixv + ndof);
  S.rhs.assign(rhs, rhs + ndof);
  S.rhs_complete = is_rhs_complete != 0;
  S.sol.assign(sol, sol + ndof);
  S.matrixtype = matrixtype;
  S.ia.assign(i_sparse, i_sparse + la);
  S.ja.assign(j_sparse, j_sparse + la);
  S.a.assign(a_sparse, a_sparse + la);
  if (matrixtype != 0)  // symmetric storage: upper triangle (module_levels.f90:748-752)
    for (int k = 0; k < la; ++k)
      if (S.ia[k] > S.ja[k]) { o->err = "only the upper triangle is expected"; return 2; }
  coo_assemble(S.ia, S.ja, S.a);
  S.bc_present = false;
  for (int i = 0; i < ndof; ++i) if (S.ifix[i] != 0) S.bc_present = true;
  nodal_components(S, find_components != 0, neighbouring);
  return 0;
}

// interior and augmented solves: Cholesky factors for symmetric matrices, LU for general ones
static void a11_solve(const Sub& S, double* x) {
  if (S.matrixtype == 0) S.a11lu.solve(x);
  else S.a11.solve(x);
}
static void aug_solve(const Sub& S, double* x) {
  if (S.matrixtype == 0) S.auglu.solve(x);
  else S.aug.solve(x);
}
// yi += A_io xo (interface rows): from A_oi^T for symmetric matrices, the
// interface rows themselves for general ones
static void a21_apply_add(const Sub& S, const double* xo, double* yi) {
  if (S.matrixtype == 0) {
    for (int i = 0; i < S.ndofi; ++i) {
      double t = 0.0;
      for (int k = S.a21_ptr[i]; k < S.a21_ptr[i + 1]; ++k) t += S.a21_val[k] * xo[S.a21_col[k]];
      yi[i] += t;
    }
  } else {
    for (int io = 0; io < S.ndofo; ++io)
      for (int k = S.a12_ptr[io]; k < S.a12_ptr[io + 1]; ++k) yi[S.a12_col[k]] += S.a12_val[k] * xo[io];
  }
}

static void comm_exchange(Oracle& o, vector<vector<double>>& v, bool keep_own) {
  // upload / swap / download (module_dd.f90:11236-11551): the neighbours'
  // values on shared dofs summed in ascending neighbour order, either onto the
  // own value (keep_own) or into a zeroed buffer, as dd_comm_download does.
  int nsub = o.nsub;
  vector<vector<double>> out(nsub);
  for (int s = 0; s < nsub; ++s) out[s] = keep_own ? v[s] : vector<double>(v[s].size(), 0.0);
#pragma omp parallel for schedule(dynamic) num_threads(o.nthreads)
  for (int s = 0; s < nsub; ++s) {
    auto& S = o.subs[s];
    for (size_t a = 0; a < S.iadj.size(); ++a) {
      const vector<double>& vt = v[S.iadj[a] - 1];
      for (int k = S.xch_ptr[a]; k < S.xch_ptr[a + 1]; ++k) out[s][S.xch_mine[k]] += vt[S.xch_theirs[k]];
    }
  }
  v.swap(out);
}

static void comm_exchange_add(Oracle& o, vector<vector<double>>& v) { comm_exchange(o, v, true); }

static void build_exchange_lists(Oracle& o) {
  for (auto& S : o.subs) {
    S.kdofi.assign(S.nnodi + 1, 0);
    for (int i = 0; i < S.nnodi; ++i) S.kdofi[i + 1] = S.kdofi[i] + S.nndf[S.iin[i]];
  }
#pragma omp parallel for schedule(dynamic) num_threads(o.nthreads)
  for (int s = 0; s < o.nsub; ++s) {
    auto& S = o.subs[s];
    S.xch_mine.clear(); S.xch_theirs.clear(); S.xch_ptr.assign(1, 0);
    int k = 0;
    for (size_t a = 0; a < S.iadj.size(); ++a) {
      auto& T = o.subs[S.iadj[a] - 1];
      std::unordered_map<int, int> tpos;  // global node id -> neighbour interface node index
      for (int i = 0; i < T.nnodi; ++i) tpos.emplace(T.isngn[T.iin[i]], i);
      for (int ish = 0; ish < S.nshnadj[a]; ++ish) {
        int inodi = S.ishnadj[k + ish];
        int tinodi = tpos.at(S.isngn[S.iin[inodi]]);
        int nd = S.kdofi[inodi + 1] - S.kdofi[inodi];
        for (int d = 0; d < nd; ++d) { S.xch_mine.push_back(S.kdofi[inodi] + d); S.xch_theirs.push_back(T.kdofi[tinodi] + d); }
      }
      S.xch_ptr.push_back((int)S.xch_mine.size());
      k += S.nshnadj[a];
    }
  }
}

// global coarse dofs of every coarse node and the constraint rows of every
// subdomain in CSR over its interface dofs (module_dd.f90:11011-11235, 5018-5144)
static void number_constraints(Oracle& o) {
  int ncnode = o.ncorner + o.nedge + o.nface;
  o.ncdof_of_cnode.assign(ncnode, 0);
  for (auto& S : o.subs)
    for (auto& cn : S.cnodes) o.ncdof_of_cnode[cn.global_cnode - 1] = cn.ncdof;
  vector<int> kdofc(ncnode + 1, 0);
  for (int c = 0; c < ncnode; ++c) kdofc[c + 1] = kdofc[c] + o.ncdof_of_cnode[c];
  o.ndofc = kdofc[ncnode];
  for (auto& S : o.subs) {
    S.crow_ptr.assign(1, 0); S.crow_col.clear(); S.crow_val.clear(); S.indrowc.clear();
    for (auto& cn : S.cnodes) {
      cn.igcdof.clear();
      for (int d = 0; d < cn.ncdof; ++d) cn.igcdof.push_back(kdofc[cn.global_cnode - 1] + d + 1);
      if (!cn.used) continue;
      for (int r = 0; r < cn.ncdof; ++r) {
        for (int v = 0; v < cn.nvar; ++v) {
          double val = cn.matrix[(size_t)r * cn.nvar + v];
          if (std::fabs(val) > 0.0) { S.crow_col.push_back(cn.ivsivn[v]); S.crow_val.push_back(val); }
        }
        S.crow_ptr.push_back((int)S.crow_col.size());
        S.indrowc.push_back(cn.igcdof[r]);
      }
    }
    S.nconstr = (int)S.indrowc.size();
  }
}

static void coarse_space(Oracle& o);

// explicit Schur complement of a subdomain, ndofi x ndofi row-major
// (dd_prepare_explicit_schur; the same operator as dd_multiply_by_schur)
static vector<double> dense_schur(Sub& S) {
  const int ni = S.ndofi;
  vector<vector<std::pair<int, double>>> a12c(ni);  // A_oi by interface column
  for (int io = 0; io < S.ndofo; ++io)
    for (int k = S.a12_ptr[io]; k < S.a12_ptr[io + 1]; ++k) a12c[S.a12_col[k]].push_back({io, S.a12_val[k]});
  vector<double> sd((size_t)ni * ni, 0.0), aux(S.ndofo);
  for (int c = 0; c < ni; ++c) {
    for (int k = S.a22_ptr[c]; k < S.a22_ptr[c + 1]; ++k) sd[(size_t)S.a22_col[k] * ni + c] += S.a22_val[k];
    if (S.ndofo == 0 || a12c[c].empty()) continue;
    std::fill(aux.begin(), aux.end(), 0.0);
    for (auto& e : a12c[c]) aux[e.first] = e.second;
    S.a11.solve(aux.data());
    for (int io = 0; io < S.ndofo; ++io)
      for (int k = S.a12_ptr[io]; k < S.a12_ptr[io + 1]; ++k) sd[(size_t)S.a12_col[k] * ni + c] -= S.a12_val[k] * aux[io];
  }
  for (int r = 0; r < ni; ++r)
    for (int c = r + 1; c < ni; ++c) {
      double m = 0.5 * (sd[(size_t)r * ni + c] + sd[(size_t)c * ni + r]);
      sd[(size_t)r * ni + c] = sd[(size_t)c * ni + r] = m;
    }
  return sd;
}

// M <- P M P with P = I - Q Q^T, Q (n x m) column-major orthonormal
static void project_both(int n, vector<double>& M, const vector<double>& Q, int m) {
  if (m == 0) return;
  vector<double> mq((size_t)n * m, 0.0);  // M Q, row-major n x m
  for (int r = 0; r < n; ++r)
    for (int k = 0; k < m; ++k) {
      double t = 0.0;
      for (int c = 0; c < n; ++c) t += M[(size_t)r * n + c] * Q[(size_t)k * n + c];
      mq[(size_t)r * m + k] = t;
    }
  vector<double> qmq((size_t)m * m, 0.0);  // Q^T M Q
  for (int a = 0; a < m; ++a)
    for (int b = 0; b < m; ++b) {
      double t = 0.0;
      for (int r = 0; r < n; ++r) t += Q[(size_t)a * n + r] * mq[(size_t)r * m + b];
      qmq[(size_t)a * m + b] = t;
    }
  // P M P = M - MQ Q^T - Q (MQ)^T + Q (Q^T M Q) Q^T   (M symmetric)
  vector<double> qq((size_t)n * m, 0.0);  // Q (Q^T M Q), row-major n x m
  for (int r = 0; r < n; ++r)
    for (int b = 0; b < m; ++b) {
      double t = 0.0;
      for (int a = 0; a < m; ++a) t += Q[(size_t)a * n + r] * qmq[(size_t)a * m + b];
      qq[(size_t)r * m + b] = t;
    }
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c) {
      double t = 0.0;
      for (int k = 0; k < m; ++k)
        t += -mq[(size_t)r * m + k] * Q[(size_t)k * n + c] - Q[(size_t)k * n + r] * mq[(size_t)c * m + k] +
             qq[(size_t)r * m + k] * Q[(size_t)k * n + c];
      M[(size_t)r * n + c] += t;
    }
}

// Adaptive face constraints (adaptivity_solve_eigenvectors, module_adaptivity.f90:296-2514,
// with the pair operators of adaptivity_mvecmult, :2560-3023).  For each face shared by
// subdomains i and j, on the space of both interfaces (n = ndofi_i + ndofi_j):
//   D  = [C_i  -C_j] on the coarse dofs common to i and j; P the orthogonal projection onto null(D)
//   E  = weighted average on the common dofs (weights rho_i/(rho_i + rho_j)), I - E zero elsewhere
//   A  = P (I-E)^T S (I-E) P,   B = P S P + t (I - P),  S = diag(S_i, S_j), t = max |diag S|
// and the largest min(10, ncommon_dofs - ncommon_coarse) eigenvalues of A v = lambda B v are
// computed exactly (B restricted to its range: null(S) within null(D) carries no information).
// Eigenvectors with lambda >= tau give constraints A v restricted to the face dofs; each face's
// rows [arithmetic average; adaptive] are orthonormalised by pivoted QR with the 1 % rule
// (dd_orthogonalize_constraints, module_dd.f90:4637-4760) and given to both subdomains.
static void adaptivity(Oracle& o, const vector<vector<double>>& rho) {
  const int nsub = o.nsub;
  number_constraints(o);
  vector<vector<double>> sd(nsub);
  std::string errs;
#pragma omp parallel for schedule(dynamic) num_threads(o.nthreads)
  for (int s = 0; s < nsub; ++s) sd[s] = dense_schur(o.subs[s]);
  // pairs = faces, ordered by global coarse node (dd_create_pairs, module_dd.f90:10785-11008)
  std::map<int, vector<std::pair<int, int>>> faces;
  for (int s = 0; s < nsub; ++s)
    for (int c = 0; c < (int)o.subs[s].cnodes.size(); ++c)
      if (o.subs[s].cnodes[c].itype == 1) faces[o.subs[s].cnodes[c].global_cnode].push_back({s, c});
  o.pairs.clear();
  vector<std::array<int, 2>> pcn;
  for (auto& f : faces) {
    if (f.second.size() != 2) throw std::runtime_error("a face not shared by exactly two subdomains");
    o.pairs.push_back({f.first, f.second[0].first, f.second[1].first});
    pcn.push_back({f.second[0].second, f.second[1].second});
  }
  const int npair = (int)o.pairs.size();
  o.pair_eigs.assign(npair, {});
  o.pair_nadaptive.assign(npair, 0);
  o.face_ncdof.assign(npair, 0);
  vector<vector<double>> cons(npair);  // adaptive rows over the face dofs of the first subdomain
  vector<double> est_loc(npair, 0.0);
#pragma omp parallel for schedule(dynamic) num_threads(o.nthreads)
  for (int p = 0; p < npair; ++p) {
    try {
      const int si = o.pairs[p][1], sj = o.pairs[p][2];
      Sub& A = o.subs[si];
      Sub& Bq = o.subs[sj];
      const int ni = A.ndofi, nj = Bq.ndofi, n = ni + nj;
      // common interface dofs
      std::unordered_map<int, int> jnode;
      for (int i = 0; i < Bq.nnodi; ++i) jnode[Bq.isngn[Bq.iin[i]]] = i;
      vector<std::array<int, 2>> cd;
      vector<double> wa, wb;
      for (int i = 0; i < A.nnodi; ++i) {
        auto it = jnode.find(A.isngn[A.iin[i]]);
        if (it == jnode.end()) continue;
        for (int d = 0; d < A.nndf[A.iin[i]]; ++d) {
          int a = A.kdofi[i] + d, b = ni + Bq.kdofi[it->second] + d;
          double ra = rho[si][a], rb = rho[sj][b - ni];
          cd.push_back({a, b});
          wa.push_back(ra / (ra + rb));
          wb.push_back(rb / (ra + rb));
        }
      }
      // D^T columns: coarse dofs common to both
      std::unordered_map<int, int> jrow;
      for (int r = 0; r < Bq.nconstr; ++r) jrow[Bq.indrowc[r]] = r;
      vector<vector<double>> dcol;
      for (int r = 0; r < A.nconstr; ++r) {
        auto it = jrow.find(A.indrowc[r]);
        if (it == jrow.end()) continue;
        vector<double> v(n, 0.0);
        for (int k = A.crow_ptr[r]; k < A.crow_ptr[r + 1]; ++k) v[A.crow_col[k]] += A.crow_val[k];
        for (int k = Bq.crow_ptr[it->second]; k < Bq.crow_ptr[it->second + 1]; ++k)
          v[ni + Bq.crow_col[k]] -= Bq.crow_val[k];
        dcol.push_back(v);
      }
      const int m = (int)dcol.size();
      const int neig = std::min(10, (int)cd.size() - m);
      if (neig <= 0) { est_loc[p] = 1.0; continue; }
      // orthonormal basis of range(D^T): Gram-Schmidt, twice
      vector<double> q;
      int mq = 0;
      for (auto& v : dcol) {
        for (int pass = 0; pass < 2; ++pass)
          for (int k = 0; k < mq; ++k) {
            double t = 0.0;
            for (int r = 0; r < n; ++r) t += q[(size_t)k * n + r] * v[r];
            for (int r = 0; r < n; ++r) v[r] -= t * q[(size_t)k * n + r];
          }
        double nv = 0.0;
        for (int r = 0; r < n; ++r) nv += v[r] * v[r];
        nv = std::sqrt(nv);
        if (nv < 1e-12) continue;
        for (int r = 0; r < n; ++r) q.push_back(v[r] / nv);
        ++mq;
      }
      // S = diag(S_i, S_j)
      vector<double> Sm((size_t)n * n, 0.0);
      for (int r = 0; r < ni; ++r)
        for (int c = 0; c < ni; ++c) Sm[(size_t)r * n + c] = sd[si][(size_t)r * ni + c];
      for (int r = 0; r < nj; ++r)
        for (int c = 0; c < nj; ++c) Sm[(size_t)(ni + r) * n + ni + c] = sd[sj][(size_t)r * nj + c];
      double t = 0.0;
      for (int r = 0; r < n; ++r) t = std::max(t, std::fabs(Sm[(size_t)r * n + r]));
      // A = P E^T S E P
      vector<double> F((size_t)n * n, 0.0), Am((size_t)n * n, 0.0);
      for (size_t k = 0; k < cd.size(); ++k) {
        const int a = cd[k][0], b = cd[k][1];
        for (int r = 0; r < n; ++r) {
          F[(size_t)r * n + a] = (1.0 - wa[k]) * Sm[(size_t)r * n + a] - wa[k] * Sm[(size_t)r * n + b];
          F[(size_t)r * n + b] = -wb[k] * Sm[(size_t)r * n + a] + (1.0 - wb[k]) * Sm[(size_t)r * n + b];
        }
      }
      for (size_t k = 0; k < cd.size(); ++k) {
        const int a = cd[k][0], b = cd[k][1];
        for (int c = 0; c < n; ++c) {
          Am[(size_t)a * n + c] = (1.0 - wa[k]) * F[(size_t)a * n + c] - wa[k] * F[(size_t)b * n + c];
          Am[(size_t)b * n + c] = -wb[k] * F[(size_t)a * n + c] + (1.0 - wb[k]) * F[(size_t)b * n + c];
        }
      }
      for (int r = 0; r < n; ++r)
        for (int c = r + 1; c < n; ++c) {
          double mm = 0.5 * (Am[(size_t)r * n + c] + Am[(size_t)c * n + r]);
          Am[(size_t)r * n + c] = Am[(size_t)c * n + r] = mm;
        }
      project_both(n, Am, q, mq);
      // B = P S P + t (I - P)
      vector<double> Bm = Sm;
      project_both(n, Bm, q, mq);
      for (int k = 0; k < mq; ++k)  // I - P = Q Q^T
        for (int r = 0; r < n; ++r)
          for (int c = 0; c < n; ++c) Bm[(size_t)r * n + c] += t * q[(size_t)k * n + r] * q[(size_t)k * n + c];
      // B = U diag(sig) U^T; keep sig > 1e-12 max; V = U_keep sig^-1/2; H = V^T A V
      vector<double> sig, U;
      vector<double> bcopy = Bm;
      sym_eig(n, bcopy, sig, U);
      const double smax = sig.empty() ? 0.0 : sig.back();
      vector<int> keep;
      for (int k = 0; k < n; ++k) if (sig[k] > 1e-12 * smax) keep.push_back(k);
      const int nk = (int)keep.size();
      vector<double> V((size_t)n * nk);
      for (int r = 0; r < n; ++r)
        for (int k = 0; k < nk; ++k) V[(size_t)r * nk + k] = U[(size_t)r * n + keep[k]] / std::sqrt(sig[keep[k]]);
      vector<double> AV((size_t)n * nk, 0.0), H((size_t)nk * nk, 0.0);
      for (int r = 0; r < n; ++r)
        for (int c = 0; c < n; ++c) {
          const double arc = Am[(size_t)r * n + c];
          if (arc == 0.0) continue;
          for (int k = 0; k < nk; ++k) AV[(size_t)r * nk + k] += arc * V[(size_t)c * nk + k];
        }
      for (int a = 0; a < nk; ++a)
        for (int b = 0; b < nk; ++b) {
          double tt = 0.0;
          for (int r = 0; r < n; ++r) tt += V[(size_t)r * nk + a] * AV[(size_t)r * nk + b];
          H[(size_t)a * nk + b] = tt;
        }
      for (int a = 0; a < nk; ++a)
        for (int b = a + 1; b < nk; ++b) {
          double mm = 0.5 * (H[(size_t)a * nk + b] + H[(size_t)b * nk + a]);
          H[(size_t)a * nk + b] = H[(size_t)b * nk + a] = mm;
        }
      vector<double> lam, Y;
      sym_eig(nk, H, lam, Y);
      const int ne = std::min(neig, nk);
      vector<double> ev(ne);
      for (int k = 0; k < ne; ++k) ev[k] = lam[nk - 1 - k];
      int nad = 0;
      for (double l : ev) if (l >= o.adaptive_tau) ++nad;
      est_loc[p] = ne > 0 ? (nad < ne ? ev[nad] : ev[nad - 1]) : 1.0;
      o.pair_eigs[p] = ev;
      o.pair_nadaptive[p] = nad;
      // constraints A v over the face dofs of subdomain i
      const Cnode& cf = A.cnodes[pcn[p][0]];
      vector<double> rows((size_t)nad * cf.nvar, 0.0);
      for (int k = 0; k < nad; ++k) {
        const int col = nk - 1 - k;
        vector<double> v(n, 0.0), av(n, 0.0);
        for (int r = 0; r < n; ++r) {
          double tt = 0.0;
          for (int a = 0; a < nk; ++a) tt += V[(size_t)r * nk + a] * Y[(size_t)a * nk + col];
          v[r] = tt;
        }
        for (int r = 0; r < n; ++r) {
          double tt = 0.0;
          for (int c = 0; c < n; ++c) tt += Am[(size_t)r * n + c] * v[c];
          av[r] = tt;
        }
        for (int vv = 0; vv < cf.nvar; ++vv) rows[(size_t)k * cf.nvar + vv] = av[cf.ivsivn[vv]];
      }
      cons[p] = rows;
    } catch (std::exception& e) {
#pragma omp critical
      errs = e.what();
    }
  }
  if (!errs.empty()) throw std::runtime_error(errs);
  o.adaptivity_est = -1.0;
  for (double e : est_loc) o.adaptivity_est = std::max(o.adaptivity_est, e);
  // load, orthonormalise and share the face constraints
  for (int p = 0; p < npair; ++p) {
    Sub& A = o.subs[o.pairs[p][1]];
    Sub& Bq = o.subs[o.pairs[p][2]];
    Cnode& ci = A.cnodes[pcn[p][0]];
    Cnode& cj = Bq.cnodes[pcn[p][1]];
    const int nvar = ci.nvar;
    const int nad = o.pair_nadaptive[p];
    const int ncol = ci.ncdof + nad;
    vector<double> mcol((size_t)nvar * ncol);
    for (int r = 0; r < ci.ncdof; ++r)
      for (int v = 0; v < nvar; ++v) mcol[(size_t)r * nvar + v] = ci.matrix[(size_t)r * nvar + v];
    for (int r = 0; r < nad; ++r)
      for (int v = 0; v < nvar; ++v) mcol[(size_t)(ci.ncdof + r) * nvar + v] = cons[p][(size_t)r * nvar + v];
    int nvalid = 0;
    vector<double> qb = pivoted_orthonormal_basis(nvar, ncol, mcol, nvalid);
    // face dof order of j by global dof
    std::unordered_map<int, int> gpos;
    for (int v = 0; v < cj.nvar; ++v) gpos[Bq.isvgvn[Bq.iivsvn[cj.ivsivn[v]]]] = v;
    ci.matrix.assign((size_t)nvalid * nvar, 0.0);
    cj.matrix.assign((size_t)nvalid * nvar, 0.0);
    for (int r = 0; r < nvalid; ++r)
      for (int v = 0; v < nvar; ++v) {
        const double val = qb[(size_t)r * nvar + v];
        ci.matrix[(size_t)r * nvar + v] = val;
        cj.matrix[(size_t)r * nvar + gpos.at(A.isvgvn[A.iivsvn[ci.ivsivn[v]]])] = val;
      }
    ci.ncdof = cj.ncdof = nvalid;
    ci.used = cj.used = nvalid > 0;
    o.face_ncdof[p] = nvalid;
  }
  number_constraints(o);
}

// reduced right-hand side g = f_i - A_io A_oo^-1 f_o, assembled (module_dd.f90:6995-7257)
static void reduced_rhs(Oracle& oo) {
    Oracle* o = &oo;
    const int nsub = o->nsub;
    vector<vector<double>> g(nsub);
#pragma omp parallel for schedule(dynamic) num_threads(o->nthreads)
    for (int s = 0; s < nsub; ++s) {
      auto& S = o->subs[s];
      vector<double> rhs = S.rhs;
      if (S.rhs_complete) for (int i = 0; i < S.ndofi; ++i) rhs[S.iivsvn[i]] *= S.wi[i];
      if (S.bc_present) {
        vector<double> bcw = S.bc;
        for (int i = 0; i < S.ndofi; ++i) bcw[S.iivsvn[i]] *= S.wi[i];
        for (int i = 0; i < S.ndof; ++i) { if (S.ifix[i]) rhs[i] = 0.0; rhs[i] += bcw[i]; }
      }
      S.solo.assign(S.ndofo, 0.0);
      for (int i = 0; i < S.ndofo; ++i) S.solo[i] = rhs[S.iovsvn[i]];
      if (S.ndofo > 0) a11_solve(S, S.solo.data());
      g[s].assign(S.ndofi, 0.0);
      a21_apply_add(S, S.solo.data(), g[s].data());
      for (int i = 0; i < S.ndofi; ++i) g[s][i] = rhs[S.iivsvn[i]] - g[s][i];
    }
    comm_exchange_add(*o, g);
    for (int s = 0; s < nsub; ++s) o->subs[s].g = g[s];
}

Oracle::~Oracle() { delete lev2; }

// recursive coordinate bisection of the level-1 subdomain centroids into
// nparts level-2 subdomains: split along the longest extent, halves by count
// (ties by subdomain index); stands in for the METIS division of the reference
static void rcb(vector<int> ids, int nparts, int first, const vector<std::array<double, 3>>& c, int ndim,
                vector<int>& part) {
  if (nparts <= 1 || ids.size() <= 1) {
    for (int id : ids) part[id] = first;
    return;
  }
  int axis = 0;
  double best = -1.0;
  for (int a = 0; a < ndim; ++a) {
    double lo = 1e300, hi = -1e300;
    for (int id : ids) { lo = std::min(lo, c[id][a]); hi = std::max(hi, c[id][a]); }
    if (hi - lo > best * (1.0 + 1e-12)) { best = hi - lo; axis = a; }
  }
  std::stable_sort(ids.begin(), ids.end(), [&](int x, int y) {
    return c[x][axis] != c[y][axis] ? c[x][axis] < c[y][axis] : x < y;
  });
  const int k1 = nparts / 2;
  const size_t n1 = ids.size() * (size_t)k1 / (size_t)nparts;
  rcb(vector<int>(ids.begin(), ids.begin() + n1), k1, first, c, ndim, part);
  rcb(vector<int>(ids.begin() + n1, ids.end()), nparts - k1, first + k1, c, ndim, part);
}

extern "C" int oracle_setup(void* h, int use_corner_constraints, int use_arithmetic_constraints, int weights_type);

// the level-2 problem (levels_prepare_standard_level, module_levels.f90:1297-3000):
// nodes = level-1 coarse nodes (corner: its node, edge / face: mean of the glob's
// nodes), elements = level-1 subdomains with their coarse matrices Phi^T A Phi
static void build_level2(Oracle& o) {

  const int nsub = o.nsub;
  const int ndim = o.subs[0].ndim;
  const int ncnode = o.ncorner + o.nedge + o.nface;
  vector<int> ncd(ncnode, 0), kdc(ncnode, -1);
  vector<std::array<double, 3>> xc(ncnode, {0.0, 0.0, 0.0}), cent(nsub, {0.0, 0.0, 0.0});
  for (int s = 0; s < nsub; ++s) {
    const Sub& S = o.subs[s];
    for (int i = 0; i < S.nnod; ++i)
      for (int d = 0; d < ndim; ++d) cent[s][d] += S.xyz[(size_t)d * S.nnod + i] / S.nnod;
    for (const Cnode& cn : S.cnodes) {
      if (!cn.used) continue;
      const int g = cn.global_cnode - 1;
      if (kdc[g] >= 0) continue;
      ncd[g] = cn.ncdof;
      kdc[g] = cn.igcdof[0] - 1;
      for (int in : cn.insin)
        for (int d = 0; d < ndim; ++d) xc[g][d] += S.xyz[(size_t)d * S.nnod + S.iin[in]] / (double)cn.insin.size();
    }
  }
  vector<int> part(nsub, 0), ids(nsub);
  std::iota(ids.begin(), ids.end(), 0);
  rcb(ids, o.nsub2, 0, cent, ndim, part);
  Oracle* o2 = new Oracle;
  o2->nsub = o.nsub2;
  o2->nthreads = o.nthreads;
  o2->subs.resize(o.nsub2);
  o.lev2 = o2;
  for (int t2 = 0; t2 < o.nsub2; ++t2) {
    vector<int> elems;
    for (int s = 0; s < nsub; ++s) if (part[s] == t2) elems.push_back(s);
    if (elems.empty()) throw std::runtime_error("empty level-2 subdomain");
    std::map<int, int> loc;
    for (int s : elems)
      for (const Cnode& cn : o.subs[s].cnodes) if (cn.used) loc.emplace(cn.global_cnode - 1, 0);
    int nn = 0, nd = 0;
    vector<int> kd, isngn, nndf, isvgvn, isegn, inet, nnet, ia, ja;
    vector<double> xyz, a;
    for (auto& kv : loc) {
      kv.second = nn++;
      isngn.push_back(kv.first);
      nndf.push_back(ncd[kv.first]);
      kd.push_back(nd);
      nd += ncd[kv.first];
    }
    isvgvn.resize(nd);
    xyz.assign((size_t)nn * ndim, 0.0);
    for (auto& kv : loc) {
      for (int d = 0; d < ncd[kv.first]; ++d) isvgvn[kd[kv.second] + d] = kdc[kv.first] + d;
      for (int d = 0; d < ndim; ++d) xyz[(size_t)d * nn + kv.second] = xc[kv.first][d];
    }
    for (int s : elems) {
      const Sub& S = o.subs[s];
      isegn.push_back(s);
      vector<int> rowdof;
      int cnt = 0;
      for (const Cnode& cn : S.cnodes) {
        if (!cn.used) continue;
        const int l = loc.at(cn.global_cnode - 1);
        inet.push_back(l);
        ++cnt;
        for (int d = 0; d < cn.ncdof; ++d) rowdof.push_back(kd[l] + d);
      }
      nnet.push_back(cnt);
      const int nc = (int)rowdof.size();
      for (int r = 0; r < nc; ++r)
        for (int c = 0; c < nc; ++c) {
          const int i = rowdof[r], j = rowdof[c];
          if (i < j || r == c) {
            ia.push_back(i);
            ja.push_back(j);
            a.push_back(r == c ? S.coarsem[(size_t)r * nc + r]
                               : 0.5 * (S.coarsem[(size_t)r * nc + c] + S.coarsem[(size_t)c * nc + r]));
          }
        }
    }
    vector<int> ifix(nd, 0);
    vector<double> zero(nd, 0.0);
    if (oracle_upload(o2, t2, (int)elems.size(), nn, nd, ndim, inet.data(), (int)inet.size(), nnet.data(),
                      nndf.data(), isngn.data(), isvgvn.data(), isegn.data(), xyz.data(), ifix.data(), zero.data(),
                      zero.data(), 1, zero.data(), 1, (int)a.size(), ia.data(), ja.data(), a.data(), 1, 1) != 0)
      throw std::runtime_error("level-2 upload: " + o2->err);
  }
  if (oracle_setup(o2, o.setup_corner, o.setup_arith, o.setup_weights) != 0)
    throw std::runtime_error("level-2 setup: " + o2->err);
}

int oracle_setup(void* h, int use_corner_constraints, int use_arithmetic_constraints, int weights_type) {
  {
    auto* og = static_cast<Oracle*>(h);
    const bool gen = !og->subs.empty() && og->subs[0].matrixtype == 0;
    if (gen && (og->adaptive || og->nlevels == 3)) {
      og->err = "adaptive constraints and three levels need a symmetric matrix";
      return 1;
    }
  }
  auto* o = static_cast<Oracle*>(h);
  try {
    int nsub = o->nsub;
    int meshdim = o->subs[0].ndim;
    create_neighbouring(*o);
    build_exchange_lists(*o);
    create_globs(*o, use_corner_constraints != 0, meshdim);
    // ---- BC elimination (module_dd.f90:1081-1256, module_sm.f90:431-600)
    vector<vector<double>> bci(nsub);
    for (int s = 0; s < nsub; ++s) {
      auto& S = o->subs[s];
      S.bc.assign(S.ndof, 0.0);
      if (S.bc_present) {
        vector<char> diag_fixed(S.ndof, 0);
        S.fx_i.clear(); S.fx_j.clear(); S.fx_v.clear();
        const bool sym = S.matrixtype != 0;
        for (size_t k = 0; k < S.ia.size(); ++k) {
          int i = S.ia[k], j = S.ja[k];
          if (S.ifix[i] || (sym && S.ifix[j])) { S.fx_i.push_back(i); S.fx_j.push_back(j); S.fx_v.push_back(S.a[k]); }
          if (i != j) {
            // a fixed row moves into the rhs only in symmetric storage (module_sm.f90:528-541)
            if (sym && S.ifix[i] && S.fixv[i] != 0.0 && S.a[k] != 0.0 && !S.ifix[j]) S.bc[j] -= S.a[k] * S.fixv[i];
            if (S.ifix[j] && S.fixv[j] != 0.0 && S.a[k] != 0.0 && !S.ifix[i]) S.bc[i] -= S.a[k] * S.fixv[j];
            if (S.ifix[i] || S.ifix[j]) S.a[k] = 0.0;
          } else if (S.ifix[i]) {
            if (std::fabs(S.a[k]) < 1e-16) S.a[k] = 1.0;
            if (S.fixv[i] != 0.0) S.bc[i] += S.a[k] * S.fixv[i];
            diag_fixed[i] = 1;
          }
        }
        for (int i = 0; i < S.ndof; ++i)
          if (S.ifix[i] > 0 && !diag_fixed[i]) {
            S.ia.push_back(i); S.ja.push_back(i); S.a.push_back(1.0);
            S.bc[i] += S.fixv[i];
          }
        coo_assemble(S.ia, S.ja, S.a);
      }
      bci[s].assign(S.ndofi, 0.0);
      for (int i = 0; i < S.ndofi; ++i) bci[s][i] = S.bc[S.iivsvn[i]];
    }
    {
      vector<vector<double>> nb = bci;
      comm_exchange(*o, nb, false);
      for (int s = 0; s < nsub; ++s) {
        auto& S = o->subs[s];
        for (int i = 0; i < S.ndofi; ++i) S.bc[S.iivsvn[i]] += nb[s][i];
      }
    }
    // ---- weights (module_dd.f90:11554-11722)
    vector<vector<double>> rho(nsub);
    for (int s = 0; s < nsub; ++s) {
      auto& S = o->subs[s];
      rho[s].assign(S.ndofi, 1.0);
      if (weights_type == 1) {
        vector<double> dg(S.ndof, 0.0);
        for (size_t k = 0; k < S.ia.size(); ++k) if (S.ia[k] == S.ja[k]) dg[S.ia[k]] += S.a[k];
        for (int i = 0; i < S.ndofi; ++i) { rho[s][i] = dg[S.iivsvn[i]]; if (rho[s][i] == 0.0) rho[s][i] = 1.0; }
      } else if (weights_type != 0) {
        throw std::runtime_error("weights type not supported by the oracle");
      }
    }
    {
      vector<vector<double>> aux = rho;
      comm_exchange(*o, aux, false);
      for (int s = 0; s < nsub; ++s) {
        auto& S = o->subs[s];
        S.wi.resize(S.ndofi);
        for (int i = 0; i < S.ndofi; ++i) S.wi[i] = rho[s][i] / (rho[s][i] + aux[s][i]);
      }
    }
    // ---- constraints and coarse dofs (module_levels.f90:2690-2740, module_dd.f90:11011-11235, 5018-5144)
    for (int s = 0; s < nsub; ++s) {
      auto& S = o->subs[s];
      if (use_corner_constraints) load_arithmetic_constraints(S, 3);
      if (use_arithmetic_constraints) { load_arithmetic_constraints(S, 2); load_arithmetic_constraints(S, 1); }
    }
    number_constraints(*o);
    // ---- per-subdomain factorisations (module_dd.f90:3983-4295, 5211-5799)
    std::string errs;
#pragma omp parallel for schedule(dynamic) num_threads(o->nthreads)
    for (int s = 0; s < nsub; ++s) {
      try {
        auto& S = o->subs[s];
        if (S.matrixtype == 0) csr_from_full(S.ndof, S.ia, S.ja, S.a, S.f_ptr, S.f_col, S.f_val);
        else sym_csr_from_upper(S.ndof, S.ia, S.ja, S.a, S.f_ptr, S.f_col, S.f_val);
        // blocks
        vector<int> mo(S.ndof, -1), mi(S.ndof, -1);
        for (int i = 0; i < S.ndofo; ++i) mo[S.iovsvn[i]] = i;
        for (int i = 0; i < S.ndofi; ++i) mi[S.iivsvn[i]] = i;
        S.a12_ptr.assign(S.ndofo + 1, 0); S.a12_col.clear(); S.a12_val.clear();
        S.a22_ptr.assign(S.ndofi + 1, 0); S.a22_col.clear(); S.a22_val.clear();
        int b11 = 0;
        for (int io = 0; io < S.ndofo; ++io) {
          int r = S.iovsvn[io];
          for (int k = S.f_ptr[r]; k < S.f_ptr[r + 1]; ++k) {
            int c = S.f_col[k];
            if (mi[c] >= 0) { S.a12_col.push_back(mi[c]); S.a12_val.push_back(S.f_val[k]); }
            else b11 = std::max(b11, std::abs(io - mo[c]));
          }
          S.a12_ptr[io + 1] = (int)S.a12_col.size();
        }
        S.a21_ptr.assign(S.ndofi + 1, 0); S.a21_col.clear(); S.a21_val.clear();
        for (int ii = 0; ii < S.ndofi; ++ii) {
          int r = S.iivsvn[ii];
          for (int k = S.f_ptr[r]; k < S.f_ptr[r + 1]; ++k) {
            int c = S.f_col[k];
            if (mi[c] >= 0) { S.a22_col.push_back(mi[c]); S.a22_val.push_back(S.f_val[k]); }
            else if (S.matrixtype == 0) { S.a21_col.push_back(mo[c]); S.a21_val.push_back(S.f_val[k]); }
          }
          S.a22_ptr[ii + 1] = (int)S.a22_col.size();
          S.a21_ptr[ii + 1] = (int)S.a21_col.size();
        }
        if (S.matrixtype == 0) {
          S.a11lu.n = S.ndofo; S.a11lu.b = b11;
          S.a11lu.v.assign((size_t)S.ndofo * (2 * b11 + 1), 0.0);
          for (int io = 0; io < S.ndofo; ++io) {
            int r = S.iovsvn[io];
            for (int k = S.f_ptr[r]; k < S.f_ptr[r + 1]; ++k) {
              int c = S.f_col[k];
              if (mo[c] >= 0) S.a11lu.at(io, mo[c]) += S.f_val[k];
            }
          }
          if (S.ndofo > 0) S.a11lu.factor();
        } else {
          S.a11.n = S.ndofo; S.a11.b = b11;
          S.a11.v.assign((size_t)S.ndofo * (b11 + 1), 0.0);
          for (int io = 0; io < S.ndofo; ++io) {
            int r = S.iovsvn[io];
            for (int k = S.f_ptr[r]; k < S.f_ptr[r + 1]; ++k) {
              int c = S.f_col[k];
              if (mo[c] >= 0 && mo[c] <= io) S.a11.at(io, mo[c]) += S.f_val[k];
            }
          }
          if (S.ndofo > 0) S.a11.factor();
        }
        // augmented system: corner dofs shifted by their own diagonal
        int baug = 0;
        for (int r = 0; r < S.ndof; ++r)
          for (int k = S.f_ptr[r]; k < S.f_ptr[r + 1]; ++k) baug = std::max(baug, std::abs(r - S.f_col[k]));
        if (S.matrixtype == 0) {
          S.auglu.n = S.ndof; S.auglu.b = baug;
          S.auglu.v.assign((size_t)S.ndof * (2 * baug + 1), 0.0);
          for (int r = 0; r < S.ndof; ++r)
            for (int k = S.f_ptr[r]; k < S.f_ptr[r + 1]; ++k) S.auglu.at(r, S.f_col[k]) += S.f_val[k];
          for (auto& cn : S.cnodes)
            if (cn.itype == 3 && cn.used)
              for (int v : cn.ivsivn) { int d = S.iivsvn[v]; S.auglu.at(d, d) *= 2.0; }
          S.auglu.factor();
        } else {
          S.aug.n = S.ndof; S.aug.b = baug;
          S.aug.v.assign((size_t)S.ndof * (baug + 1), 0.0);
          for (int r = 0; r < S.ndof; ++r)
            for (int k = S.f_ptr[r]; k < S.f_ptr[r + 1]; ++k)
              if (S.f_col[k] <= r) S.aug.at(r, S.f_col[k]) += S.f_val[k];
          for (auto& cn : S.cnodes)
            if (cn.itype == 3 && cn.used)
              for (int v : cn.ivsivn) { int d = S.iivsvn[v]; S.aug.at(d, d) *= 2.0; }
          S.aug.factor();
        }
      } catch (std::exception& e) {
#pragma omp critical
        errs = e.what();
      }
    }
    if (!errs.empty()) throw std::runtime_error(errs);
    // ---- adaptive face constraints (module_levels.f90:2826-2938)
    if (o->adaptive) adaptivity(*o, rho);
    coarse_space(*o);
    // ---- level 2 of three (module_levels.f90:1297-3000)
    o->setup_corner = use_corner_constraints;
    o->setup_arith = use_arithmetic_constraints;
    o->setup_weights = weights_type;
    delete o->lev2;
    o->lev2 = nullptr;
    if (o->nlevels == 3) build_level2(*o);
    reduced_rhs(*o);
    o->setup_done = true;
  } catch (std::exception& e) {
    o->err = e.what();
    return 1;
  }
  return 0;
}

// coarse basis of one subdomain for its current constraints (module_dd.f90:5211-5799):
// Y = A_r^-1 C^T, G = C Y, Phi = Y G^-1, coarse matrix Phi^T A Phi
static void coarse_basis(Sub& S) {
        int nc = S.nconstr;
        const bool gen = S.matrixtype == 0;
        S.yaug.assign((size_t)S.ndof * nc, 0.0);
        for (int c = 0; c < nc; ++c) {
          double* y = &S.yaug[(size_t)c * S.ndof];
          for (int k = S.crow_ptr[c]; k < S.crow_ptr[c + 1]; ++k) y[S.iivsvn[S.crow_col[k]]] += S.crow_val[k];
          aug_solve(S, y);
        }
        if (gen) {  // adjoint problem A^T for the dual basis (module_dd.f90:5687-5757)
          S.ydual.assign((size_t)S.ndof * nc, 0.0);
          for (int c = 0; c < nc; ++c) {
            double* y = &S.ydual[(size_t)c * S.ndof];
            for (int k = S.crow_ptr[c]; k < S.crow_ptr[c + 1]; ++k) y[S.iivsvn[S.crow_col[k]]] += S.crow_val[k];
            S.auglu.solve_t(y);
          }
        }
        S.gchol.assign((size_t)nc * nc, 0.0);
        for (int r = 0; r < nc; ++r)
          for (int c = 0; c < nc; ++c) {
            double t = 0.0;
            for (int k = S.crow_ptr[r]; k < S.crow_ptr[r + 1]; ++k) t += S.crow_val[k] * S.yaug[(size_t)c * S.ndof + S.iivsvn[S.crow_col[k]]];
            S.gchol[(size_t)r * nc + c] = t;
          }
        if (!gen) {
          for (int r = 0; r < nc; ++r)
            for (int c = r + 1; c < nc; ++c) {
              double m = 0.5 * (S.gchol[(size_t)r * nc + c] + S.gchol[(size_t)c * nc + r]);
              S.gchol[(size_t)r * nc + c] = S.gchol[(size_t)c * nc + r] = m;
            }
          if (nc > 0) dense_chol(S.gchol, nc);
        } else if (nc > 0) {
          dense_lu(S.gchol, nc, S.gpiv);
        }
        // coarse basis: Phi = Y G^{-1}   (solve with RHS [0; I], module_dd.f90:5592-5607);
        // for a general matrix also the dual basis Phi_dual = Y_dual G^{-T}
        auto basis = [&](const vector<double>& y, bool trans) {
          vector<double> phi((size_t)S.ndof * nc, 0.0);
          for (int c = 0; c < nc; ++c) {
            vector<double> e(nc, 0.0); e[c] = 1.0;
            if (gen) dense_lu_solve(S.gchol, nc, S.gpiv, e.data(), trans);
            else dense_chol_solve(S.gchol, nc, e.data());
            for (int i = 0; i < S.ndof; ++i) {
              double t = 0.0;
              for (int q = 0; q < nc; ++q) t += y[(size_t)q * S.ndof + i] * e[q];
              phi[(size_t)c * S.ndof + i] = t;
            }
          }
          return phi;
        };
        vector<double> phi = basis(S.yaug, false);
        vector<double> phid = gen ? basis(S.ydual, true) : phi;
        S.phisi.assign((size_t)S.ndofi * nc, 0.0);
        for (int c = 0; c < nc; ++c)
          for (int i = 0; i < S.ndofi; ++i) S.phisi[(size_t)c * S.ndofi + i] = phi[(size_t)c * S.ndof + S.iivsvn[i]];
        if (gen) {
          S.phisi_dual.assign((size_t)S.ndofi * nc, 0.0);
          for (int c = 0; c < nc; ++c)
            for (int i = 0; i < S.ndofi; ++i)
              S.phisi_dual[(size_t)c * S.ndofi + i] = phid[(size_t)c * S.ndof + S.iivsvn[i]];
        }
        // coarse matrix Phi_dual^T A Phi (Phi^T A Phi for symmetric matrices)
        S.coarsem.assign((size_t)nc * nc, 0.0);
        vector<double> aphi(S.ndof);
        for (int c = 0; c < nc; ++c) {
          csr_mult(S.f_ptr, S.f_col, S.f_val, &phi[(size_t)c * S.ndof], aphi.data(), S.ndof);
          for (int r = 0; r < nc; ++r) {
            double t = 0.0;
            for (int i = 0; i < S.ndof; ++i) t += phid[(size_t)r * S.ndof + i] * aphi[i];
            S.coarsem[(size_t)r * nc + c] = t;
          }
        }
}

// coarse bases of all subdomains, then the coarse problem
// (module_levels.f90:3001-3170): assemble the upper triangle, factor
static void coarse_space(Oracle& oo) {
    Oracle* o = &oo;
    std::string errs;
#pragma omp parallel for schedule(dynamic) num_threads(o->nthreads)
    for (int s = 0; s < o->nsub; ++s) {
      try {
        coarse_basis(o->subs[s]);
      } catch (std::exception& e) {
#pragma omp critical
        errs = e.what();
      }
    }
    if (!errs.empty()) throw std::runtime_error(errs);
    int n = o->ndofc;
    o->coarse_chol.assign((size_t)n * n, 0.0);
    const bool gen = !o->subs.empty() && o->subs[0].matrixtype == 0;
    for (auto& S : o->subs) {
      int nc = S.nconstr;
      if (gen) {  // all entries of the general local coarse matrices
        for (int i = 0; i < nc; ++i)
          for (int j = 0; j < nc; ++j)
            o->coarse_chol[(size_t)(S.indrowc[i] - 1) * n + (S.indrowc[j] - 1)] += S.coarsem[(size_t)i * nc + j];
        continue;
      }
      for (int j = 0; j < nc; ++j)
        for (int i = 0; i <= j; ++i) {
          int gi = S.indrowc[i] - 1, gj = S.indrowc[j] - 1;
          double v = S.coarsem[(size_t)i * nc + j];
          int r = std::max(gi, gj), c = std::min(gi, gj);
          o->coarse_chol[(size_t)r * n + c] += v;
        }
    }
    if (gen) {
      if (n > 0) dense_lu(o->coarse_chol, n, o->coarse_piv);
      return;
    }
    for (int r = 0; r < n; ++r)
      for (int c = r + 1; c < n; ++c) o->coarse_chol[(size_t)r * n + c] = o->coarse_chol[(size_t)c * n + r];
    if (n > 0) dense_chol(o->coarse_chol, n, o->nthreads);
}

// y = S x per subdomain (module_dd.f90:6564-6699), then exchange
static void sm_apply(Oracle& o, vector<vector<double>>& x, vector<vector<double>>& y) {
#pragma omp parallel for schedule(dynamic) num_threads(o.nthreads)
  for (int s = 0; s < o.nsub; ++s) {
    auto& S = o.subs[s];
    vector<double> aux1(S.ndofo, 0.0);
    for (int io = 0; io < S.ndofo; ++io) {
      double t = 0.0;
      for (int k = S.a12_ptr[io]; k < S.a12_ptr[io + 1]; ++k) t += S.a12_val[k] * x[s][S.a12_col[k]];
      aux1[io] = t;
    }
    if (S.ndofo > 0) a11_solve(S, aux1.data());
    vector<double> aux2(S.ndofi, 0.0);
    a21_apply_add(S, aux1.data(), aux2.data());
    y[s].assign(S.ndofi, 0.0);
    for (int i = 0; i < S.ndofi; ++i) {
      double t = 0.0;
      for (int k = S.a22_ptr[i]; k < S.a22_ptr[i + 1]; ++k) t += S.a22_val[k] * x[s][S.a22_col[k]];
      y[s][i] = t - aux2[i];
    }
  }
  comm_exchange_add(o, y);
}

static void pc_apply(Oracle& o, vector<vector<double>>& r, vector<vector<double>>& z);

// One BDDC application on level 2 for the level-1 coarse residual rc (global
// coarse dofs, 0-based): interior solves of the level-2 subdomains, reduced rhs
// on the level-2 interface (rhs given complete: interface values weighted),
// the level-2 preconditioner, interior resolve (levels_corsub_standard_level,
// levels_solve_last_level, levels_add_standard_level, module_levels.f90:3849-4250).
static vector<double> level2_apply(Oracle& o2, const vector<double>& rc) {
  const int nsub = o2.nsub;
  vector<vector<double>> g(nsub), z(nsub), f(nsub), solo(nsub);
  for (int s = 0; s < nsub; ++s) {
    auto& S = o2.subs[s];
    f[s].resize(S.ndof);
    for (int d = 0; d < S.ndof; ++d) f[s][d] = rc[S.isvgvn[d]];
    for (int i = 0; i < S.ndofi; ++i) f[s][S.iivsvn[i]] *= S.wi[i];
    solo[s].assign(S.ndofo, 0.0);
    for (int io = 0; io < S.ndofo; ++io) solo[s][io] = f[s][S.iovsvn[io]];
    if (S.ndofo > 0) S.a11.solve(solo[s].data());
    g[s].assign(S.ndofi, 0.0);
    for (int io = 0; io < S.ndofo; ++io)
      for (int k = S.a12_ptr[io]; k < S.a12_ptr[io + 1]; ++k) g[s][S.a12_col[k]] += S.a12_val[k] * solo[s][io];
    for (int i = 0; i < S.ndofi; ++i) g[s][i] = f[s][S.iivsvn[i]] - g[s][i];
  }
  comm_exchange_add(o2, g);
  pc_apply(o2, g, z);
  vector<double> uc(rc.size(), 0.0);
  for (int s = 0; s < nsub; ++s) {
    auto& S = o2.subs[s];
    vector<double> uo(S.ndofo);
    for (int io = 0; io < S.ndofo; ++io) {
      double t = 0.0;
      for (int k = S.a12_ptr[io]; k < S.a12_ptr[io + 1]; ++k) t += S.a12_val[k] * z[s][S.a12_col[k]];
      uo[io] = f[s][S.iovsvn[io]] - t;
    }
    if (S.ndofo > 0) S.a11.solve(uo.data());
    for (int io = 0; io < S.ndofo; ++io) uc[S.isvgvn[S.iovsvn[io]]] = uo[io];
    for (int i = 0; i < S.ndofi; ++i) uc[S.isvgvn[S.iivsvn[i]]] = z[s][i];
  }
  return uc;
}

// z = M r (module_levels.f90:3627-3703, 3707-3846, 4029-4061, 4252-4346)
static void pc_apply(Oracle& o, vector<vector<double>>& r, vector<vector<double>>& z) {
  int n = o.ndofc;
  vector<double> rc(n, 0.0);
  vector<vector<double>> rcs(o.nsub);
#pragma omp parallel for schedule(dynamic) num_threads(o.nthreads)
  for (int s = 0; s < o.nsub; ++s) {
    auto& S = o.subs[s];
    int nc = S.nconstr;
    vector<double> aux(S.ndofi);
    for (int i = 0; i < S.ndofi; ++i) aux[i] = S.wi[i] * r[s][i];
    rcs[s].assign(nc, 0.0);
    // restriction with the dual basis for a general matrix (dd_phisi_dual_apply, module_dd.f90:6126-6206)
    const vector<double>& phr = S.matrixtype == 0 ? S.phisi_dual : S.phisi;
    for (int c = 0; c < nc; ++c) {
      double t = 0.0;
      for (int i = 0; i < S.ndofi; ++i) t += phr[(size_t)c * S.ndofi + i] * aux[i];
      rcs[s][c] = t;
    }
    // constrained Neumann solve with interface RHS, interior zero
    vector<double> f(S.ndof, 0.0);
    for (int i = 0; i < S.ndofi; ++i) f[S.iivsvn[i]] = aux[i];
    aug_solve(S, f.data());
    vector<double> mu(nc, 0.0);
    for (int c = 0; c < nc; ++c) {
      double t = 0.0;
      for (int k = S.crow_ptr[c]; k < S.crow_ptr[c + 1]; ++k) t += S.crow_val[k] * f[S.iivsvn[S.crow_col[k]]];
      mu[c] = t;
    }
    if (nc > 0) {
      if (S.matrixtype == 0) dense_lu_solve(S.gchol, nc, S.gpiv, mu.data(), false);
      else dense_chol_solve(S.gchol, nc, mu.data());
    }
    z[s].assign(S.ndofi, 0.0);
    for (int i = 0; i < S.ndofi; ++i) {
      int d = S.iivsvn[i];
      double t = f[d];
      for (int c = 0; c < nc; ++c) t -= S.yaug[(size_t)c * S.ndof + d] * mu[c];
      z[s][i] = t;
    }
  }
  for (int s = 0; s < o.nsub; ++s) {
    auto& S = o.subs[s];
    for (int c = 0; c < S.nconstr; ++c) rc[S.indrowc[c] - 1] += rcs[s][c];
  }
  if (n > 0) {
    if (o.lev2) rc = level2_apply(*o.lev2, rc);
    else if (!o.coarse_piv.empty()) dense_lu_solve(o.coarse_chol, n, o.coarse_piv, rc.data(), false);
    else dense_chol_solve(o.coarse_chol, n, rc.data());
  }
#pragma omp parallel for schedule(dynamic) num_threads(o.nthreads)
  for (int s = 0; s < o.nsub; ++s) {
    auto& S = o.subs[s];
    for (int c = 0; c < S.nconstr; ++c) {
      double u = rc[S.indrowc[c] - 1];
      for (int i = 0; i < S.ndofi; ++i) z[s][i] += S.phisi[(size_t)c * S.ndofi + i] * u;
    }
    for (int i = 0; i < S.ndofi; ++i) z[s][i] *= S.wi[i];
  }
  comm_exchange_add(o, z);
}

static double dotw(Oracle& o, vector<vector<double>>& a, vector<vector<double>>& b) {
  double t = 0.0;
  for (int s = 0; s < o.nsub; ++s) {
    auto& S = o.subs[s];
    double ts = 0.0;
    for (int i = 0; i < S.ndofi; ++i) ts += a[s][i] * S.wi[i] * b[s][i];
    t += ts;
  }
  return t;
}

static void fix_bc_dual(Oracle& o, vector<vector<double>>& v) {
  for (int s = 0; s < o.nsub; ++s) {
    auto& S = o.subs[s];
    if (!S.bc_present) continue;
    for (int i = 0; i < S.ndofi; ++i) if (S.ifix[S.iivsvn[i]]) v[s][i] = 0.0;
  }
}

// largest eigenvalue of a symmetric tridiagonal matrix by Sturm bisection
// (stands in for LAPACK DSTEV in module_krylov.f90:2061-2118)
static double tridiag_max_eig(const vector<double>& d, const vector<double>& e) {
  int n = (int)d.size();
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < n; ++i) {
    double r = (i > 0 ? std::fabs(e[i - 1]) : 0.0) + (i < n - 1 ? std::fabs(e[i]) : 0.0);
    lo = std::min(lo, d[i] - r); hi = std::max(hi, d[i] + r);
  }
  auto count_below = [&](double x) {
    int cnt = 0; double q = 1.0;
    for (int i = 0; i < n; ++i) {
      q = d[i] - x - (i > 0 ? e[i - 1] * e[i - 1] / q : 0.0);
      if (q == 0.0) q = -1e-300;
      if (q < 0) cnt++;
    }
    return cnt;
  };
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (count_below(mid) >= n) hi = mid; else lo = mid;
    if (hi - lo <= 1e-15 * std::max(1.0, std::fabs(hi))) break;
  }
  return 0.5 * (lo + hi);
}

static void postprocess(Oracle& o, vector<vector<double>>& x);

static int solve_pcg(Oracle* o, double tol, int maxit, int ndecrmax, bool recycling, int maxvec, int* num_iter,
                     int* converged_reason, double* condition_number);

int oracle_solve(void* h, double tol, int maxit, int ndecrmax, int* num_iter, int* converged_reason,
                 double* condition_number) {
  return solve_pcg(static_cast<Oracle*>(h), tol, maxit, ndecrmax, false, 0, num_iter, converged_reason,
                   condition_number);
}

// PCG with Krylov recycling (module_krylov.f90:313-484, 663-726): the stored
// S-orthonormal directions V (W = S V) project the initial residual
// (x += V V^T r, r -= S V V^T r) and every new direction is S-orthogonalised
// against them by classical Gram-Schmidt twice (krylov_orthogonalize_icgs,
// :1930-1961) before it is stored while there is room.
int oracle_solve_recycling(void* h, double tol, int maxit, int ndecrmax, int recycling, int maxvec, int* num_iter,
                           int* converged_reason, double* condition_number) {
  return solve_pcg(static_cast<Oracle*>(h), tol, maxit, ndecrmax, recycling != 0, maxvec, num_iter,
                   converged_reason, condition_number);
}

// new loads and initial guess of a subdomain after setup (bddcml_change_subdomain_data
// with the same Dirichlet data), then the reduced rhs again
int oracle_new_loads(void* h, int isub, const double* rhs, const double* sol) {
  auto* o = static_cast<Oracle*>(h);
  if (!o->setup_done || isub < 0 || isub >= o->nsub) { o->err = "bad call"; return 1; }
  auto& S = o->subs[isub];
  S.rhs.assign(rhs, rhs + S.ndof);
  S.sol.assign(sol, sol + S.ndof);
  reduced_rhs(*o);
  return 0;
}

static int solve_pcg(Oracle* o, double tol, int maxit, int ndecrmax, bool recycling, int maxvec, int* num_iter,
                     int* converged_reason, double* condition_number) {
  if (!o->setup_done) { o->err = "setup not done"; return 1; }
  int nsub = o->nsub;
  vector<vector<double>> x(nsub), r(nsub), p(nsub), ap(nsub), z(nsub);
  // initial data (module_levels.f90:4374-4440)
  for (int s = 0; s < nsub; ++s) {
    auto& S = o->subs[s];
    vector<double> sol = S.sol;
    if (S.bc_present) for (int i = 0; i < S.ndof; ++i) if (S.ifix[i]) sol[i] = S.fixv[i];
    x[s].resize(S.ndofi);
    for (int i = 0; i < S.ndofi; ++i) x[s][i] = sol[S.iivsvn[i]];
    r[s] = S.g;
  }
  fix_bc_dual(*o, r);
  o->relres_hist.clear();
  *num_iter = 0; *converged_reason = 0; *condition_number = 1.0;
  double normrhs = std::sqrt(dotw(*o, r, r));
  if (normrhs == 0.0) return 0;
  sm_apply(*o, x, ap);
  fix_bc_dual(*o, ap);
  for (int s = 0; s < nsub; ++s) for (size_t i = 0; i < r[s].size(); ++i) r[s][i] -= ap[s][i];
  double normres0 = std::sqrt(dotw(*o, r, r));
  if (normres0 == 0.0) return 0;
  vector<double> diag(maxit + 1, 0.0), subdiag(maxit, 0.0);
  int nw = 0;
  if (recycling && o->rc_cap == 0) o->rc_cap = std::max(0, maxvec);
  auto combine = [&](const vector<vector<vector<double>>>& basis, const vector<double>& c,
                     vector<vector<double>>& out, double sign) {
    for (size_t j = 0; j < c.size(); ++j)
      for (int s = 0; s < nsub; ++s)
        for (size_t i = 0; i < out[s].size(); ++i) out[s][i] += sign * c[j] * basis[j][s][i];
  };
  bool projected_done = false;
  if (recycling && !o->rcv.empty()) {
    // x += V V^T r, r -= S V V^T r (module_krylov.f90:373-452)
    vector<double> c(o->rcv.size());
    for (size_t j = 0; j < c.size(); ++j) c[j] = dotw(*o, o->rcv[j], r);
    for (int s = 0; s < nsub; ++s) z[s].assign(r[s].size(), 0.0);
    combine(o->rcv, c, z, 1.0);
    for (int s = 0; s < nsub; ++s)
      for (size_t i = 0; i < x[s].size(); ++i) x[s][i] += z[s][i];
    sm_apply(*o, z, ap);
    for (int s = 0; s < nsub; ++s)
      for (size_t i = 0; i < r[s].size(); ++i) r[s][i] -= ap[s][i];
    fix_bc_dual(*o, r);
    const double relres = std::sqrt(dotw(*o, r, r)) / normres0;
    if (relres < tol) projected_done = true;  // no iteration needed
  }
  if (normres0 != 0.0 && !projected_done) {
    pc_apply(*o, r, p);
    double rmp = dotw(*o, r, p);
    int ndecr = 0;
    double lastres = 1.0;
    for (int iter = 1; iter <= maxit; ++iter) {
      if (recycling && !o->rcv.empty())
        for (int pass = 0; pass < 2; ++pass) {  // p -= V W^T p, twice
          vector<double> c(o->rcv.size());
          for (size_t j = 0; j < c.size(); ++j) c[j] = dotw(*o, o->rcw[j], p);
          combine(o->rcv, c, p, -1.0);
        }
      sm_apply(*o, p, ap);
      double pap = dotw(*o, p, ap);
      if (recycling && (int)o->rcv.size() < o->rc_cap) {
        const double sc = 1.0 / std::sqrt(pap);
        vector<vector<double>> v = p, w = ap;
        for (int s = 0; s < nsub; ++s)
          for (size_t i = 0; i < v[s].size(); ++i) { v[s][i] *= sc; w[s][i] *= sc; }
        o->rcv.push_back(v);
        o->rcw.push_back(w);
      }
      double alpha = rmp / pap;
      for (int s = 0; s < nsub; ++s)
        for (size_t i = 0; i < x[s].size(); ++i) { x[s][i] += alpha * p[s][i]; r[s][i] -= alpha * ap[s][i]; }
      double normres = std::sqrt(dotw(*o, r, r));
      double relres = normres / normres0;
      o->relres_hist.push_back(relres);
      if (relres < tol) { nw = iter - 1; *num_iter = iter; *converged_reason = 0; break; }
      if (iter == maxit) { nw = iter - 1; *num_iter = iter; *converged_reason = -1; break; }
      if (relres < lastres) ndecr = 0;
      else if (++ndecr >= ndecrmax) { nw = iter - 1; *num_iter = iter; *converged_reason = -2; break; }
      lastres = relres;
      pc_apply(*o, r, z);
      double rmpold = rmp;
      rmp = dotw(*o, r, z);
      double beta = rmp / rmpold;
      for (int s = 0; s < nsub; ++s)
        for (size_t i = 0; i < p[s].size(); ++i) p[s][i] = z[s][i] + beta * p[s][i];
      diag[iter - 1] += 1.0 / alpha;
      diag[iter] = beta / alpha;
      subdiag[iter - 1] = beta >= 0.0 ? -std::sqrt(beta) / alpha : 0.0;
    }
    if (nw > 1) {
      vector<double> d(diag.begin(), diag.begin() + nw), e(subdiag.begin(), subdiag.begin() + nw - 1);
      *condition_number = tridiag_max_eig(d, e);
    } else {
      *condition_number = 1.0;
    }
  }
  postprocess(*o, x);
  return 0;
}

// interior values from the interface solution x
// (module_levels.f90:4510-4576, module_dd.f90:6811-6932)
static void postprocess(Oracle& oo, vector<vector<double>>& x) {
  Oracle* o = &oo;
  int nsub = o->nsub;
#pragma omp parallel for schedule(dynamic) num_threads(o->nthreads)
  for (int s = 0; s < nsub; ++s) {
    auto& S = o->subs[s];
    vector<double> u(S.ndof, 0.0);
    if (S.ndofo > 0) {
      vector<double> rhs = S.rhs;
      if (S.bc_present) for (int i = 0; i < S.ndof; ++i) { if (S.ifix[i]) rhs[i] = 0.0; rhs[i] += S.bc[i]; }
      vector<double> aux1(S.ndofo);
      for (int io = 0; io < S.ndofo; ++io) {
        double t = 0.0;
        for (int k = S.a12_ptr[io]; k < S.a12_ptr[io + 1]; ++k) t += S.a12_val[k] * x[s][S.a12_col[k]];
        aux1[io] = rhs[S.iovsvn[io]] - t;
      }
      a11_solve(S, aux1.data());
      for (int io = 0; io < S.ndofo; ++io) u[S.iovsvn[io]] += aux1[io];
    }
    for (int i = 0; i < S.ndofi; ++i) u[S.iivsvn[i]] += x[s][i];
    S.sol = u;
  }
}

// BiCGSTAB (method 1, module_krylov.f90:948-1505) and steepest descent
// (method 2, module_krylov.f90:1508-1840); method -1 takes the defaults of
// module_bddcml.f90:515-520 (BiCGSTAB, tol 1e-6, maxit 1000, ndecrmax 30).
// Residuals are relative to the norm of r0 = g - S x0.  cond is -1: neither
// method estimates it.  Returns 2 when steepest descent stalls for ndecrmax
// iterations, which the reference treats as an error (module_krylov.f90:1801-1812).
int oracle_solve_method(void* h, int method, double tol, int maxit, int ndecrmax, int* num_iter,
                        int* converged_reason, double* condition_number) {
  if (method == 0) return oracle_solve(h, tol, maxit, ndecrmax, num_iter, converged_reason, condition_number);
  auto* o = static_cast<Oracle*>(h);
  if (method == -1) { method = 1; tol = 1e-6; maxit = 1000; ndecrmax = 30; }
  if (method != 1 && method != 2) { o->err = "unknown method"; return 1; }
  if (!o->setup_done) { o->err = "setup not done"; return 1; }
  const int nsub = o->nsub;
  vector<vector<double>> x(nsub), r(nsub), v(nsub), z(nsub);
  for (int s = 0; s < nsub; ++s) {
    auto& S = o->subs[s];
    vector<double> sol = S.sol;
    if (S.bc_present) for (int i = 0; i < S.ndof; ++i) if (S.ifix[i]) sol[i] = S.fixv[i];
    x[s].resize(S.ndofi);
    for (int i = 0; i < S.ndofi; ++i) x[s][i] = sol[S.iivsvn[i]];
    r[s] = S.g;
  }
  fix_bc_dual(*o, r);
  sm_apply(*o, x, v);
  for (int s = 0; s < nsub; ++s) for (size_t i = 0; i < r[s].size(); ++i) r[s][i] -= v[s][i];
  fix_bc_dual(*o, r);
  o->relres_hist.clear();
  *num_iter = 0; *converged_reason = -1; *condition_number = -1.0;
  const double normrhs = std::sqrt(dotw(*o, r, r));
  if (normrhs == 0.0) { *converged_reason = 0; return 0; }
  auto axpy = [&](double a, vector<vector<double>>& xx, vector<vector<double>>& yy) {
    for (int s = 0; s < nsub; ++s) for (size_t i = 0; i < yy[s].size(); ++i) yy[s][i] += a * xx[s][i];
  };
  int ndecr = 0;
  double lastres = 1.0;
  if (method == 2) {
    vector<vector<double>> az(nsub);
    for (int iter = 1; iter <= maxit; ++iter) {
      pc_apply(*o, r, z);
      sm_apply(*o, z, az);
      const double alpha = dotw(*o, r, z) / dotw(*o, z, az);
      axpy(alpha, z, x);
      axpy(-alpha, az, r);
      fix_bc_dual(*o, r);
      const double relres = std::sqrt(dotw(*o, r, r)) / normrhs;
      o->relres_hist.push_back(relres);
      *num_iter = iter;
      if (relres < tol) { *converged_reason = 0; break; }
      if (iter == maxit) { *converged_reason = -1; break; }
      if (relres < lastres) ndecr = 0;
      else if (++ndecr >= ndecrmax) {
        *converged_reason = -2;
        o->err = "steepest descent: residual did not decrease for ndecrmax iterations";
        return 2;
      }
      lastres = relres;
    }
    postprocess(*o, x);
    return 0;
  }
  vector<vector<double>> p(nsub), y(nsub), sv(nsub), t(nsub), rs = r;
  for (int s = 0; s < nsub; ++s) { v[s].assign(r[s].size(), 0.0); p[s].assign(r[s].size(), 0.0); }
  double rhoold = 1.0, alpha = 1.0, omega = 1.0;
  for (int iter = 1; iter <= maxit; ++iter) {
    const double rho = dotw(*o, r, rs);
    const double beta = rho * alpha / (rhoold * omega);
    for (int s = 0; s < nsub; ++s)
      for (size_t i = 0; i < p[s].size(); ++i) p[s][i] = r[s][i] + beta * (p[s][i] - omega * v[s][i]);
    pc_apply(*o, p, y);
    sm_apply(*o, y, v);
    alpha = rho / dotw(*o, v, rs);
    axpy(alpha, y, x);
    sv = r;
    axpy(-alpha, v, sv);
    double relres = std::sqrt(dotw(*o, sv, sv)) / normrhs;
    *num_iter = iter;
    if (relres < tol) { o->relres_hist.push_back(relres); *converged_reason = 0; break; }
    if (relres < lastres) ndecr = 0;
    else if (++ndecr >= ndecrmax) { o->relres_hist.push_back(relres); *converged_reason = -2; break; }
    lastres = relres;
    pc_apply(*o, sv, z);
    sm_apply(*o, z, t);
    omega = dotw(*o, t, sv) / dotw(*o, t, t);
    axpy(omega, z, x);
    r = sv;
    axpy(-omega, t, r);
    relres = std::sqrt(dotw(*o, r, r)) / normrhs;
    o->relres_hist.push_back(relres);
    if (relres < tol) { *converged_reason = 0; break; }
    if (iter == maxit) { *converged_reason = -1; break; }
    if (relres < lastres) ndecr = 0;
    else if (++ndecr >= ndecrmax) { *converged_reason = -2; break; }
    lastres = relres;
    rhoold = rho;
  }
  postprocess(*o, x);
  return 0;
}

int oracle_download(void* h, int isub, double* sols, int lsols) {
  auto* o = static_cast<Oracle*>(h);
  auto& S = o->subs[isub];
  if (lsols != S.ndof) return 1;
  std::copy(S.sol.begin(), S.sol.end(), sols);
  return 0;
}

// structure summary: [ncorner, nedge, nface, ndofc, sum ndofi, sum ndofo]
void oracle_stats(void* h, int* out) {
  auto* o = static_cast<Oracle*>(h);
  long si = 0, so = 0;
  for (auto& S : o->subs) { si += S.ndofi; so += S.ndofo; }
  out[0] = o->ncorner; out[1] = o->nedge; out[2] = o->nface; out[3] = o->ndofc;
  out[4] = (int)si; out[5] = (int)so;
}

// per-subdomain: [ndofi, ndofo, nconstr, ncorner_nodes, nadj]
void oracle_sub_stats(void* h, int isub, int* out) {
  auto* o = static_cast<Oracle*>(h);
  auto& S = o->subs[isub];
  int nco = 0;
  for (auto& cn : S.cnodes) if (cn.itype == 3) nco++;
  out[0] = S.ndofi; out[1] = S.ndofo; out[2] = S.nconstr; out[3] = nco; out[4] = (int)S.iadj.size();
}

int oracle_relres_history(void* h, double* out, int lout) {
  auto* o = static_cast<Oracle*>(h);
  int n = std::min<int>(lout, (int)o->relres_hist.size());
  for (int i = 0; i < n; ++i) out[i] = o->relres_hist[i];
  return (int)o->relres_hist.size();
}

// interface weights of one subdomain (ndofi values)
int oracle_weights(void* h, int isub, double* out, int lout) {
  auto* o = static_cast<Oracle*>(h);
  auto& S = o->subs[isub];
  if (lout != S.ndofi) return 1;
  std::copy(S.wi.begin(), S.wi.end(), out);
  return 0;
}

// sorted intersection and union of two integer arrays (module_utils.f90:
// get_array_intersection 878-945, get_array_union 831-876): inputs unsorted,
// outputs sorted and without repetition; returns the number of entries.
int oracle_array_intersection(const int* a, int la, const int* b, int lb, int* out) {
  vector<int> x(a, a + la), y(b, b + lb);
  vector<int> r = sorted_intersection(x, y);
  r.erase(std::unique(r.begin(), r.end()), r.end());
  std::copy(r.begin(), r.end(), out);
  return (int)r.size();
}

int oracle_array_union(const int* a, int la, const int* b, int lb, int* out) {
  vector<int> r(a, a + la);
  r.insert(r.end(), b, b + lb);
  std::sort(r.begin(), r.end());
  r.erase(std::unique(r.begin(), r.end()), r.end());
  std::copy(r.begin(), r.end(), out);
  return (int)r.size();
}

// sum_i v1 w v2 over interface + plain sum over interior (module_dd.f90:12736-12788)
double oracle_dotprod_subdomain(void* h, int isub, const double* v1, const double* v2) {
  auto* o = static_cast<Oracle*>(h);
  auto& S = o->subs[isub];
  double t = 0.0;
  for (int i = 0; i < S.ndofi; ++i) t += v1[S.iivsvn[i]] * S.wi[i] * v2[S.iivsvn[i]];
  for (int i = 0; i < S.ndofo; ++i) t += v1[S.iovsvn[i]] * v2[S.iovsvn[i]];
  return t;
}

// the dense symmetric eigensolver on its own (a: n x n row-major), for tests
void oracle_sym_eig(int n, const double* a, double* w, double* z) {
  vector<double> m(a, a + (size_t)n * n), wv, zv;
  sym_eig(n, m, wv, zv);
  std::copy(wv.begin(), wv.end(), w);
  std::copy(zv.begin(), zv.end(), z);
}

// reactions of every subdomain after a solve (dd_compute_reactions, module_dd.f90:1258-1374):
// rea = A_fixed u over the fixed-rows matrix, neighbours' interface values added, minus the
// load on the fixed dofs; out receives subdomain isub's (ndof values)
int oracle_reactions(void* h, int isub, double* out) {
  if (!static_cast<Oracle*>(h)->subs.empty() && static_cast<Oracle*>(h)->subs[0].matrixtype == 0) {
    static_cast<Oracle*>(h)->err = "reactions are restated for symmetric storage only";
    return 1;
  }
  auto* o = static_cast<Oracle*>(h);
  const int nsub = o->nsub;
  vector<vector<double>> rea(nsub), ri(nsub);
  bool any = false;
  for (int s = 0; s < nsub; ++s) {
    auto& S = o->subs[s];
    rea[s].assign(S.ndof, 0.0);
    ri[s].assign(S.ndofi, 0.0);
    if (!S.bc_present) continue;
    any = true;
    for (size_t k = 0; k < S.fx_v.size(); ++k) {
      const int i = S.fx_i[k], j = S.fx_j[k];
      rea[s][i] += S.fx_v[k] * S.sol[j];
      if (i != j) rea[s][j] += S.fx_v[k] * S.sol[i];
    }
    if (!S.rhs_complete) for (int i = 0; i < S.ndof; ++i) if (S.ifix[i]) rea[s][i] -= S.rhs[i];
    for (int i = 0; i < S.ndofi; ++i) ri[s][i] = rea[s][S.iivsvn[i]];
  }
  if (any) {
    comm_exchange(*o, ri, false);
    for (int s = 0; s < nsub; ++s) {
      auto& S = o->subs[s];
      for (int i = 0; i < S.ndofi; ++i) rea[s][S.iivsvn[i]] += ri[s][i];
      if (S.rhs_complete && S.bc_present) for (int i = 0; i < S.ndof; ++i) if (S.ifix[i]) rea[s][i] -= S.rhs[i];
    }
  }
  std::copy(rea[isub].begin(), rea[isub].end(), out);
  return 0;
}

void oracle_set_levels(void* h, int nlevels, int nsub2) {
  auto* o = static_cast<Oracle*>(h);
  o->nlevels = nlevels;
  o->nsub2 = nsub2;
}

int oracle_recycling_size(void* h) { return (int)static_cast<Oracle*>(h)->rcv.size(); }

void oracle_set_adaptive(void* h, int on, double tau) {
  auto* o = static_cast<Oracle*>(h);
  o->adaptive = on != 0;
  o->adaptive_tau = tau;
}

// pairs of the last adaptive setup: per pair (face global cnode, isub, jsub, neig, nadaptive,
// face constraints) in info (6 ints each) and its eigenvalues (10 per pair, descending,
// unused entries 0); returns the number of pairs
int oracle_adaptive_info(void* h, int* info, double* eigs, int maxpair, double* est) {
  auto* o = static_cast<Oracle*>(h);
  const int np = (int)o->pairs.size();
  for (int p = 0; p < std::min(np, maxpair); ++p) {
    info[6 * p + 0] = o->pairs[p][0];
    info[6 * p + 1] = o->pairs[p][1];
    info[6 * p + 2] = o->pairs[p][2];
    info[6 * p + 3] = (int)o->pair_eigs[p].size();
    info[6 * p + 4] = o->pair_nadaptive[p];
    info[6 * p + 5] = o->face_ncdof[p];
    for (int k = 0; k < 10; ++k) eigs[10 * p + k] = k < (int)o->pair_eigs[p].size() ? o->pair_eigs[p][k] : 0.0;
  }
  *est = o->adaptivity_est;
  return np;
}

}  // extern "C"
