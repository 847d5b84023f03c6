// Host part of the BDDC setup: the integer and geometric work that decides
// the coarse space, plus Dirichlet elimination and interface weights.
//
// All subdomains are in this process, so sharing information comes from one
// global node -> subdomains table instead of the neighbour exchanges the
// reference performs over MPI.  The decisions themselves follow the reference
// rule by rule because they fix the coarse space, and with it the iteration
// count:
//   interface = nodes shared with another subdomain ........ module_dd.f90:8360-8470
//   glob classification by sharing signature ............... module_dd.f90:9210-9276
//   corner selection on faces (farthest / largest area) .... module_dd.f90:10017-10327
//   corner union over neighbours ........................... module_dd.f90:9296-9385
//   edges and faces, Dirichlet node removal ................ module_dd.f90:9387-9587
//   coarse numbering, owner = lowest subdomain index ....... module_dd.f90:10329-10555
//   arithmetic constraints (unscaled sums) ................. module_dd.f90:4298-4384
//   coarse dof numbering ................................... module_dd.f90:11011-11235
//   Dirichlet elimination .................................. module_sm.f90:431-600, module_dd.f90:1081-1256
//   weights rho_i / sum rho ................................ module_dd.f90:11554-11722
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <numeric>
#include <omp.h>
#include <stdexcept>
#include <functional>
#include <unordered_map>

#include "bddc_internal.hpp"

namespace bddc {

double wall_time() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// sort + merge duplicate (i,j) entries (the effect of sm_assembly,
// module_sm.f90:630-684): counting sort by row keeps the upload order inside
// a row, repeated columns are summed in that order (as a stable sort followed
// by a merge would), and the distinct columns of each short row are then
// sorted.  Scratch buffers are per thread and reused across subdomains.
void host_assemble_upper(rawvec<int>& ia, rawvec<int>& ja, rawvec<double>& a) {
  static thread_local vector<int> ptr, col, slot;
  static thread_local vector<double> val;
  const size_t n = ia.size();
  int nrow = 0, ncol = 0;
  for (size_t k = 0; k < n; ++k) { nrow = std::max(nrow, ia[k] + 1); ncol = std::max(ncol, ja[k] + 1); }
  ptr.assign(nrow + 1, 0);
  for (size_t k = 0; k < n; ++k) ptr[ia[k] + 1]++;
  for (int r = 0; r < nrow; ++r) ptr[r + 1] += ptr[r];
  col.resize(n);
  val.resize(n);
  for (size_t k = 0; k < n; ++k) {
    int q = ptr[ia[k]]++;
    col[q] = ja[k];
    val[q] = a[k];
  }
  for (int r = nrow; r > 0; --r) ptr[r] = ptr[r - 1];
  ptr[0] = 0;
  slot.assign(ncol, -1);
  int out = 0;
  for (int r = 0; r < nrow; ++r) {
    const int rs = out;
    for (int i = ptr[r]; i < ptr[r + 1]; ++i) {
      int c = col[i];
      if (slot[c] >= rs) {
        a[slot[c]] += val[i];
      } else {
        slot[c] = out;
        ia[out] = r;
        ja[out] = c;
        a[out] = val[i];
        ++out;
      }
    }
    for (int i = rs + 1; i < out; ++i) {  // insertion sort of the distinct columns
      int c = ja[i];
      double v = a[i];
      int j = i - 1;
      while (j >= rs && ja[j] > c) { ja[j + 1] = ja[j]; a[j + 1] = a[j]; --j; }
      ja[j + 1] = c;
      a[j + 1] = v;
    }
  }
  ia.resize(out); ia.shrink_to_fit();
  ja.resize(out); ja.shrink_to_fit();
  a.resize(out); a.shrink_to_fit();
}

// components of the dual mesh graph: elements are connected when they share
// at least `neighbouring` nodes; a node takes the component of the last
// element that contains it (module_dd.f90:2680-2720)
void host_nodal_components(Subdomain& s) {
  s.comp.assign(s.nnod, 1);
  if (!s.find_components || s.nelem == 0) return;
  vector<int> kinet(s.nelem + 1, 0);
  for (int e = 0; e < s.nelem; ++e) kinet[e + 1] = kinet[e] + s.nnet[e];
  vector<int> nptr(s.nnod + 1, 0);
  for (int k = 0; k < kinet[s.nelem]; ++k) nptr[s.inet[k] + 1]++;
  for (int i = 0; i < s.nnod; ++i) nptr[i + 1] += nptr[i];
  vector<int> nel(nptr[s.nnod]);
  {
    vector<int> pos(nptr.begin(), nptr.end() - 1);
    for (int e = 0; e < s.nelem; ++e)
      for (int k = kinet[e]; k < kinet[e + 1]; ++k) nel[pos[s.inet[k]]++] = e;
  }
  int thr = s.dual_graph ? std::max(1, s.neighbouring) : 1;
  vector<int> ec(s.nelem, 0), cnt(s.nelem, 0), touched, stack;
  int nc = 0;
  for (int e0 = 0; e0 < s.nelem; ++e0) {
    if (ec[e0]) continue;
    ec[e0] = ++nc;
    stack.assign(1, e0);
    while (!stack.empty()) {
      int e = stack.back();
      stack.pop_back();
      touched.clear();
      for (int k = kinet[e]; k < kinet[e + 1]; ++k)
        for (int q = nptr[s.inet[k]]; q < nptr[s.inet[k] + 1]; ++q) {
          int f = nel[q];
          if (f != e && cnt[f]++ == 0) touched.push_back(f);
        }
      for (int f : touched) {
        if (cnt[f] >= thr && !ec[f]) { ec[f] = nc; stack.push_back(f); }
        cnt[f] = 0;
      }
    }
  }
  for (int e = 0; e < s.nelem; ++e)
    for (int k = kinet[e]; k < kinet[e + 1]; ++k) s.comp[s.inet[k]] = ec[e];
}

void full_symmetric_csr(const Subdomain& s, vector<int>& ptr, vector<int>& col, vector<double>& val) {
  int n = s.ndof;
  if (s.matrixtype == 0) {  // general matrix: the assembled triplets are the rows, sorted
    ptr.assign(n + 1, 0);
    for (size_t k = 0; k < s.ia.size(); ++k) ptr[s.ia[k] + 1]++;
    for (int i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
    col.assign(s.ja.begin(), s.ja.end());
    val.assign(s.a.begin(), s.a.end());
    return;
  }
  // The assembled upper triangle is sorted by (row, column): scanning it in
  // order appends the mirrored entries of every row in increasing column
  // order, and the row's own entries (its run of equal ia, copied whole)
  // follow, so no row needs sorting.  Every slot of col and val is written:
  // resize, so that buffers a caller reuses are not cleared first.
  const int* ia = s.ia.data();
  const int* ja = s.ja.data();
  const double* av = s.a.data();
  const size_t m = s.ia.size();
  static thread_local vector<int> ustart, ulen;  // each row's run in the upper triangle
  ustart.assign(n, 0);
  ulen.assign(n, 0);
  ptr.assign(n + 1, 0);
  for (size_t k = 0; k < m;) {
    const int r = ia[k];
    size_t e = k;
    while (e < m && ia[e] == r) {
      ptr[ja[e] + 1] += ja[e] != r;  // the mirrored entry lands in row ja
      ++e;
    }
    ptr[r + 1] += (int)(e - k);
    ustart[r] = (int)k;
    ulen[r] = (int)(e - k);
    k = e;
  }
  for (int i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
  col.resize(ptr[n]);
  val.resize(ptr[n]);
  static thread_local vector<int> pos;
  pos.assign(ptr.begin(), ptr.end() - 1);
  for (size_t k = 0; k < m; ++k)
    if (ia[k] != ja[k]) { int j = ja[k]; col[pos[j]] = ia[k]; val[pos[j]++] = av[k]; }
  for (int r = 0; r < n; ++r) {
    const int k0 = ustart[r], k1 = k0 + ulen[r];
    std::copy(ja + k0, ja + k1, col.begin() + pos[r]);
    std::copy(av + k0, av + k1, val.begin() + pos[r]);
  }
}

// Interior ordering for the band factor: natural order, natural order with
// the uncoupled dofs (Dirichlet dofs whose rows and columns hold only the
// diagonal) moved to the end, or reverse Cuthill-McKee, whichever has the
// smallest half bandwidth.  The interior graph (nonzero entries only: the
// removed rows and columns of fixed dofs stay in the pattern as zeros) is kept
// as flat arrays; neighbours of a visited node are queued by increasing degree
// (stable, so ties keep the matrix order).
void host_interior_ordering(Subdomain& s, const vector<int>& f_ptr, const vector<int>& f_col,
                            const vector<double>& f_val) {
  const int no = s.ndofo;
  vector<int> mo(s.ndof, -1);
  for (int i = 0; i < no; ++i) mo[s.iovsvn[i]] = i;
  vector<int> gptr(no + 1, 0), gcol;
  gcol.reserve((size_t)no * 27);
  for (int i = 0; i < no; ++i) {
    int r = s.iovsvn[i];
    for (int k = f_ptr[r]; k < f_ptr[r + 1]; ++k) {
      int c = mo[f_col[k]];
      if (c >= 0 && c != i && f_val[k] != 0.0) gcol.push_back(c);
    }
    gptr[i + 1] = (int)gcol.size();
  }
  auto deg = [&](int v) { return gptr[v + 1] - gptr[v]; };
  vector<int> inv(no);
  auto bandwidth = [&](const vector<int>& perm) {
    for (int i = 0; i < no; ++i) inv[perm[i]] = i;
    int b = 0;
    for (int i = 0; i < no; ++i)
      for (int k = gptr[i]; k < gptr[i + 1]; ++k) b = std::max(b, std::abs(inv[i] - inv[gcol[k]]));
    return b;
  };
  vector<int> natural(no);
  std::iota(natural.begin(), natural.end(), 0);
  int bn = bandwidth(natural);
  // a Dirichlet face of the subdomain interleaves uncoupled dofs with the
  // coupled ones in natural order (16 x 15 x 15 instead of 15^3 interior nodes
  // of a 16^3 subdomain): leave them out of the band
  vector<int> coupled_first;
  coupled_first.reserve(no);
  for (int i = 0; i < no; ++i) if (deg(i) > 0) coupled_first.push_back(i);
  for (int i = 0; i < no; ++i) if (deg(i) == 0) coupled_first.push_back(i);
  const int bc = bandwidth(coupled_first);
  if (bc < bn) { natural = coupled_first; bn = bc; }
  // reverse Cuthill-McKee, each component rooted at its first node of
  // minimum degree
  vector<int> rcm;
  rcm.reserve(no);
  vector<char> seen(no, 0), vis(no, 0);
  vector<int> comp;
  comp.reserve(no);
  for (int st = 0; st < no; ++st) {
    if (seen[st]) continue;
    int start = st, mind = deg(st);
    comp.assign(1, st);
    vis[st] = 1;
    for (size_t q = 0; q < comp.size(); ++q)
      for (int k = gptr[comp[q]]; k < gptr[comp[q] + 1]; ++k) {
        int c = gcol[k];
        if (!vis[c] && !seen[c]) { vis[c] = 1; comp.push_back(c); }
      }
    for (int v : comp) if (deg(v) < mind) { mind = deg(v); start = v; }
    size_t head = rcm.size();
    rcm.push_back(start);
    seen[start] = 1;
    while (head < rcm.size()) {
      int v = rcm[head++];
      size_t b = rcm.size();
      for (int k = gptr[v]; k < gptr[v + 1]; ++k) {
        int c = gcol[k];
        if (!seen[c]) { seen[c] = 1; rcm.push_back(c); }
      }
      for (size_t i = b + 1; i < rcm.size(); ++i) {  // stable insertion sort by degree
        int x = rcm[i], dx = deg(x);
        size_t j = i;
        while (j > b && deg(rcm[j - 1]) > dx) { rcm[j] = rcm[j - 1]; --j; }
        rcm[j] = x;
      }
    }
  }
  std::reverse(rcm.begin(), rcm.end());
  int br = no ? bandwidth(rcm) : 0;
  if (br < bn) { s.operm = rcm; s.band = br; }
  else { s.operm = natural; s.band = bn; }
}

namespace {

// global node -> list of (subdomain, local node) in ascending subdomain order
struct Sharing {
  vector<int> ptr;       // size nnod_global + 1
  vector<int> sub, loc;  // entries
  int count(int g) const { return ptr[g + 1] - ptr[g]; }
};

// Each thread owns a contiguous range of global node ids and scans every
// subdomain in ascending order, so each node's list is in ascending subdomain
// order whatever the thread count.
Sharing build_sharing(const Solver& S, int nnod_global) {
  Sharing sh;
  sh.ptr.assign(nnod_global + 1, 0);
  const int nsub = (int)S.subs.size();
#pragma omp parallel
  {
    const int nt = omp_get_num_threads(), th = omp_get_thread_num();
    const int g0 = (int)((long)nnod_global * th / nt), g1 = (int)((long)nnod_global * (th + 1) / nt);
    for (int t = 0; t < nsub; ++t)
      for (int g : S.subs[t].isngn)
        if (g >= g0 && g < g1) sh.ptr[g + 1]++;
#pragma omp barrier
#pragma omp single
    {
      for (int g = 0; g < nnod_global; ++g) sh.ptr[g + 1] += sh.ptr[g];
      sh.sub.resize(sh.ptr[nnod_global]);
      sh.loc.resize(sh.ptr[nnod_global]);
    }
    vector<int> pos(sh.ptr.begin() + g0, sh.ptr.begin() + g1);
    for (int t = 0; t < nsub; ++t) {
      const auto& s = S.subs[t];
      for (int i = 0; i < s.nnod; ++i) {
        const int g = s.isngn[i];
        if (g < g0 || g >= g1) continue;
        int& q = pos[g - g0];
        sh.sub[q] = t;
        sh.loc[q++] = i;
      }
    }
  }
  return sh;
}

// Holders of each unique interface dof in ascending subdomain order: those of
// u are osub / oloc (subdomain, interface index) [optr[u], optr[u + 1]).  Each
// thread owns a range of unique dofs and scans every subdomain in order.
void owner_lists(const Solver& S, vector<int>& optr, vector<int>& osub, vector<int>& oloc) {
  const int n = S.ninterface, nsub = (int)S.subs.size();
  optr.assign(n + 1, 0);
#pragma omp parallel
  {
    const int nt = omp_get_num_threads(), th = omp_get_thread_num();
    const int u0 = (int)((long)n * th / nt), u1 = (int)((long)n * (th + 1) / nt);
    for (int t = 0; t < nsub; ++t)
      for (int u : S.subs[t].uniq)
        if (u >= u0 && u < u1) optr[u + 1]++;
#pragma omp barrier
#pragma omp single
    {
      for (int u = 0; u < n; ++u) optr[u + 1] += optr[u];
      osub.resize(optr[n]);
      oloc.resize(optr[n]);
    }
    vector<int> pos(optr.begin() + u0, optr.begin() + u1);
    for (int t = 0; t < nsub; ++t) {
      const vector<int>& uq = S.subs[t].uniq;
      for (int i = 0; i < (int)uq.size(); ++i) {
        const int u = uq[i];
        if (u < u0 || u >= u1) continue;
        int& q = pos[u - u0];
        osub[q] = t;
        oloc[q++] = i;
      }
    }
  }
}

// sharing signature of a node as seen from subdomain t: for every other
// subdomain holding the node (ascending), its index, its component of the node
// and t's own component (module_dd.f90:9160-9175 globsubs).  The signatures of
// all interface nodes of a subdomain are kept flat: node i's entries are
// e[p[i]] .. e[p[i + 1]].
struct SigTable {
  vector<int> p;
  vector<std::array<int, 3>> e;
  int size(int i) const { return p[i + 1] - p[i]; }
  bool equal(int a, int b) const {
    return std::equal(e.begin() + p[a], e.begin() + p[a + 1], e.begin() + p[b], e.begin() + p[b + 1]);
  }
  bool less(int a, int b) const {
    return std::lexicographical_compare(e.begin() + p[a], e.begin() + p[a + 1], e.begin() + p[b],
                                        e.begin() + p[b + 1]);
  }
};

SigTable signatures(const Solver& S, const Sharing& sh, int t) {
  const Subdomain& s = S.subs[t];
  SigTable st;
  st.p.assign(s.nnodi + 1, 0);
  st.e.reserve((size_t)s.nnodi * 2);
  for (int i = 0; i < s.nnodi; ++i) {
    const int g = s.isngn[s.iin[i]];
    int mycomp = 0;
    for (int q = sh.ptr[g]; q < sh.ptr[g + 1]; ++q)
      if (sh.sub[q] == t) mycomp = s.comp[sh.loc[q]];
    for (int q = sh.ptr[g]; q < sh.ptr[g + 1]; ++q) {
      const int u = sh.sub[q];
      if (u == t) continue;
      st.e.push_back({u, S.subs[u].comp[sh.loc[q]], mycomp});
    }
    st.p[i + 1] = (int)st.e.size();
  }
  return st;
}

using Sig = vector<std::array<int, 3>>;

struct SigHash {
  size_t operator()(const Sig& s) const {
    size_t h = s.size();
    for (auto& a : s) h = h * 1000003u ^ (size_t)(a[0] * 31 + a[1] * 7 + a[2]);
    return h;
  }
};

// nodes grouped by equal signature, each group in visiting order, the groups
// in the order of their first node (the lookup key is one reused buffer)
vector<vector<int>> group_by_signature(const SigTable& st, const vector<int>& nodes) {
  std::unordered_map<Sig, int, SigHash> first;
  Sig key;
  vector<vector<int>> groups;
  for (int i : nodes) {
    key.assign(st.e.begin() + st.p[i], st.e.begin() + st.p[i + 1]);
    auto it = first.find(key);
    if (it == first.end()) {
      first.emplace(key, (int)groups.size());
      groups.push_back({i});
    } else {
      groups[it->second].push_back(i);
    }
  }
  return groups;
}

}  // namespace

// bc = the recorded elimination applied to the current fixed values
static void host_replay_bc(Subdomain& s) {
  s.bc.assign(s.ndof, 0.0);
  for (size_t e = 0; e < s.bcx_tgt.size(); ++e) {
    const double f = s.fixv[s.bcx_src[e]];
    if (f != 0.0) s.bc[s.bcx_tgt[e]] += s.bcx_val[e] * f;
  }
}

// interface values of bc: own value plus the other holders' values in
// ascending subdomain order (upload / swap / download, module_dd.f90:1200-1255)
static void host_interface_bc(Solver& S) {
  const int nsub = (int)S.subs.size();
  vector<int> optr, osub, oloc;
  owner_lists(S, optr, osub, oloc);
  vector<vector<double>> bci(nsub);
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    bci[t].resize(s.ndofi);
    for (int i = 0; i < s.ndofi; ++i) bci[t][i] = s.bc[s.iivsvn[i]];
  }
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    for (int i = 0; i < s.ndofi; ++i) {
      const int u = s.uniq[i];
      double acc = 0.0;
      for (int q = optr[u]; q < optr[u + 1]; ++q) if (osub[q] != t) acc += bci[osub[q]][oloc[q]];
      s.bc[s.iivsvn[i]] += acc;
    }
  }
}

void host_new_data(Solver& S) {
  const int nsub = (int)S.subs.size();
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    if (s.bc_present) host_replay_bc(s);
    else s.bc.assign(s.ndof, 0.0);
  }
  host_interface_bc(S);
}

void host_reactions(Solver& S) {
  const int nsub = (int)S.subs.size();
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    s.rea.assign(s.ndof, 0.0);
    if (!s.bc_present) continue;
    // symmetric product with the fixed-rows matrix (upper triangle stored)
    for (size_t k = 0; k < s.fxr_v.size(); ++k) {
      const int i = s.fxr_i[k], j = s.fxr_j[k];
      s.rea[i] += s.fxr_v[k] * s.sol[j];
      if (i != j) s.rea[j] += s.fxr_v[k] * s.sol[i];
    }
    if (!s.rhs_complete)
      for (int i = 0; i < s.ndof; ++i) if (s.ifix[i]) s.rea[i] -= s.rhs[i];
  }
  // neighbours' interface values added (dd_comm_upload / swapdata / download)
  vector<double> sum(S.ninterface, 0.0);
  for (auto& s : S.subs)
    if (s.bc_present)
      for (int i = 0; i < s.ndofi; ++i) sum[s.uniq[i]] += s.rea[s.iivsvn[i]];
  bool any = false;
  for (auto& s : S.subs) any = any || s.bc_present;
  if (!any) return;
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    for (int i = 0; i < s.ndofi; ++i) s.rea[s.iivsvn[i]] = sum[s.uniq[i]];
    if (s.rhs_complete && s.bc_present)
      for (int i = 0; i < s.ndof; ++i) if (s.ifix[i]) s.rea[i] -= s.rhs[i];
  }
}

void host_constraint_rows(Solver& S) {
  const int nsub = (int)S.subs.size();
  const int ncnode = S.ncorner + S.nedge + S.nface;
  vector<int> nndfc(ncnode, -1);
  for (auto& s : S.subs)
    for (auto& cn : s.cnodes) {
      int& slot = nndfc[cn.global_number - 1];
      if (slot >= 0 && slot != cn.ncdof) throw Error{ERR_NUMERIC, "inconsistent coarse node dof count"};
      slot = cn.ncdof;
    }
  vector<int> kdofc(ncnode + 1, 0);
  for (int c = 0; c < ncnode; ++c) kdofc[c + 1] = kdofc[c] + std::max(0, nndfc[c]);
  S.ndofc = kdofc[ncnode];
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    s.c_ptr.assign(1, 0); s.c_col.clear(); s.c_val.clear(); s.indrowc.clear();
    for (auto& cn : s.cnodes) {
      if (!cn.used) continue;
      if (!cn.matrix.empty()) {  // explicit rows
        const int nv = (int)cn.idofi.size();
        for (int d = 0; d < cn.ncdof; ++d) {
          for (int v = 0; v < nv; ++v) {
            const double val = cn.matrix[(size_t)d * nv + v];
            if (val != 0.0) { s.c_col.push_back(cn.idofi[v]); s.c_val.push_back(val); }
          }
          s.c_ptr.push_back((int)s.c_col.size());
          s.indrowc.push_back(kdofc[cn.global_number - 1] + d);
        }
      } else if (cn.itype == 3) {
        for (int d = 0; d < cn.ncdof; ++d) {
          s.c_col.push_back(cn.idofi[d]); s.c_val.push_back(1.0);
          s.c_ptr.push_back((int)s.c_col.size());
          s.indrowc.push_back(kdofc[cn.global_number - 1] + d);
        }
      } else {
        for (int d = 0; d < cn.ncdof; ++d) {  // row d: ones on the d-th dof of every node
          for (int i : cn.inodi) {
            int nd = s.iin[i];
            if (d < s.nndf[nd]) { s.c_col.push_back(s.kdofi[i] + d); s.c_val.push_back(1.0); }
          }
          s.c_ptr.push_back((int)s.c_col.size());
          s.indrowc.push_back(kdofc[cn.global_number - 1] + d);
        }
      }
    }
    s.nconstr = (int)s.indrowc.size();
  }
  S.stats.ndofc = S.ndofc;
}

void host_setup(Solver& S) {
  int nsub = (int)S.subs.size();
  for (int t = 0; t < nsub; ++t)
    if (!S.subs[t].loaded) throw Error{ERR_ARGUMENT, "subdomain " + std::to_string(t) + " was not uploaded"};
  int nnod_global = 0, ndof_global = 0;
  for (auto& s : S.subs) {
    for (int g : s.isngn) nnod_global = std::max(nnod_global, g + 1);
    for (int g : s.isvgvn) ndof_global = std::max(ndof_global, g + 1);
  }

  // ---- assembly of the uploaded triplets, mesh components and Dirichlet
  // elimination on each subdomain matrix (module_sm.f90:431-600, 630-684)
  double tt = wall_time();
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    if (!s.assembled) { host_assemble_upper(s.ia, s.ja, s.a); s.assembled = true; }
    host_nodal_components(s);
    s.bc.assign(s.ndof, 0.0);
    s.bcx_tgt.clear(); s.bcx_src.clear(); s.bcx_val.clear();
    s.bc_present = false;
    for (int i = 0; i < s.ndof; ++i) if (s.ifix[i] != 0) s.bc_present = true;
    if (!s.bc_present) continue;
    // fixed rows and columns are removed, the diagonal kept (set to 1 when
    // below 1e-16, module_sm.f90:547-561); what they contributed is recorded
    auto record = [&](int tgt, int src, double v) {
      s.bcx_tgt.push_back(tgt); s.bcx_src.push_back(src); s.bcx_val.push_back(v);
    };
    vector<char> diag_fixed(s.ndof, 0);
    s.fxr_i.clear(); s.fxr_j.clear(); s.fxr_v.clear();
    const bool sym = s.matrixtype != 0;  // general storage: only fixed columns feed the rhs
    for (size_t k = 0; k < s.ia.size(); ++k) {
      int i = s.ia[k], j = s.ja[k];
      if (s.ifix[i] || (sym && s.ifix[j])) { s.fxr_i.push_back(i); s.fxr_j.push_back(j); s.fxr_v.push_back(s.a[k]); }
      if (i != j) {
        if (sym && s.ifix[i] && s.a[k] != 0.0 && !s.ifix[j]) record(j, i, -s.a[k]);
        if (s.ifix[j] && s.a[k] != 0.0 && !s.ifix[i]) record(i, j, -s.a[k]);
        if (s.ifix[i] || s.ifix[j]) s.a[k] = 0.0;
      } else if (s.ifix[i]) {
        if (std::fabs(s.a[k]) < 1e-16) s.a[k] = 1.0;
        record(i, i, s.a[k]);
        diag_fixed[i] = 1;
      }
    }
    bool added = false;
    for (int i = 0; i < s.ndof; ++i)
      if (s.ifix[i] > 0 && !diag_fixed[i]) {
        s.ia.push_back(i); s.ja.push_back(i); s.a.push_back(1.0);
        record(i, i, 1.0);
        added = true;
      }
    host_replay_bc(s);
    if (added) host_assemble_upper(s.ia, s.ja, s.a);
  }
  S.stats.t_host_assemble = wall_time() - tt;
  tt = wall_time();

  // ---- interface and neighbours
  Sharing sh = build_sharing(S, nnod_global);
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    s.kdof.assign(s.nnod, 0);
    for (int i = 1; i < s.nnod; ++i) s.kdof[i] = s.kdof[i - 1] + s.nndf[i - 1];
    s.iin.clear(); s.iivsvn.clear(); s.iovsvn.clear();
    std::vector<char> isadj(nsub, 0);
    for (int i = 0; i < s.nnod; ++i) {
      int g = s.isngn[i];
      if (sh.count(g) > 1) {
        s.iin.push_back(i);
        for (int d = 0; d < s.nndf[i]; ++d) s.iivsvn.push_back(s.kdof[i] + d);
        for (int q = sh.ptr[g]; q < sh.ptr[g + 1]; ++q) if (sh.sub[q] != t) isadj[sh.sub[q]] = 1;
      } else {
        for (int d = 0; d < s.nndf[i]; ++d) s.iovsvn.push_back(s.kdof[i] + d);
      }
    }
    s.nnodi = (int)s.iin.size();
    s.ndofi = (int)s.iivsvn.size();
    s.ndofo = (int)s.iovsvn.size();
    s.kdofi.assign(s.nnodi + 1, 0);
    for (int i = 0; i < s.nnodi; ++i) s.kdofi[i + 1] = s.kdofi[i] + s.nndf[s.iin[i]];
    s.adj.clear();
    for (int u = 0; u < nsub; ++u) if (isadj[u]) s.adj.push_back(u);
  }

  S.stats.t_host_iface = wall_time() - tt;
  tt = wall_time();
  // ---- pass 1: glob classification and corner selection, per subdomain
  vector<char> corner_node(nnod_global, 0);  // union of all subdomains' corner choices
  vector<vector<int>> pass1_corners(nsub);
  vector<SigTable> sigt(nsub);  // kept for pass 2: the components do not change in between
  int meshdim = S.subs.empty() ? 3 : S.subs[0].ndim;
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    int nnodi = s.nnodi;
    sigt[t] = signatures(S, sh, t);
    const SigTable& st = sigt[t];
    vector<int> type(nnodi, 0);
    {
      vector<int> all(nnodi);
      std::iota(all.begin(), all.end(), 0);
      for (const auto& grp : group_by_signature(st, all))
        for (int i : grp) type[i] = st.size(i) == 1 ? 1 : (grp.size() > 1 ? 2 : 3);
    }
    if (S.prm.use_corner) {
      // per neighbour sharing a face: up to four extreme points of each
      // component of the shared node set (module_dd.f90:10017-10327)
      // nodes shared with each neighbour (its position in s.adj), in node order
      vector<vector<std::pair<int, int>>> shared(s.adj.size());  // (global id, inodi)
      for (int i = 0; i < nnodi; ++i)
        for (int q = st.p[i]; q < st.p[i + 1]; ++q) {
          const size_t k = std::lower_bound(s.adj.begin(), s.adj.end(), st.e[q][0]) - s.adj.begin();
          shared[k].emplace_back(s.isngn[s.iin[i]], i);
        }
      for (size_t ka = 0; ka < s.adj.size(); ++ka) {
        const int u = s.adj[ka];
        // shared nodes with u, ascending global id
        vector<std::pair<int, int>>& shn = shared[ka];
        std::sort(shn.begin(), shn.end());
        bool face = false;
        for (auto& p : shn) if (type[p.second] == 1) { face = true; break; }
        if (!face) continue;
        int m = (int)shn.size();
        vector<int> myc(m), adc(m);
        for (int q = 0; q < m; ++q) {
          int i = shn[q].second;
          for (int r = st.p[i]; r < st.p[i + 1]; ++r)
            if (st.e[r][0] == u) { adc[q] = st.e[r][1]; myc[q] = st.e[r][2]; }
        }
        auto renumber = [](vector<int>& v) {  // values -> their rank among the distinct values, from 1
          vector<int> u(v);
          std::sort(u.begin(), u.end());
          u.erase(std::unique(u.begin(), u.end()), u.end());
          for (int& x : v) x = (int)(std::lower_bound(u.begin(), u.end(), x) - u.begin()) + 1;
          return (int)u.size();
        };
        renumber(myc);
        int nadc = renumber(adc);
        vector<int> ic(m);
        for (int q = 0; q < m; ++q) ic[q] = (myc[q] - 1) * nadc + adc[q];
        int nic = renumber(ic);
        for (int c = 1; c <= nic; ++c) {
          vector<int> members;
          for (int q = 0; q < m; ++q) if (ic[q] == c) members.push_back(q);
          int mm = (int)members.size();
          vector<double> x(3 * mm, 0.0);
          for (int q = 0; q < mm; ++q) {
            int nd = s.iin[shn[members[q]].second];
            for (int d = 0; d < s.ndim; ++d) x[3 * q + d] = s.xyz[(size_t)d * s.nnod + nd];
          }
          int pick[4] = {-1, -1, -1, -1};
          auto farthest = [&](int base) {
            double best = -1.0;
            int loc = 0;
            for (int q = 0; q < mm; ++q) {
              double dd = 0.0;
              for (int d = 0; d < s.ndim; ++d) { double df = x[3 * q + d] - x[3 * base + d]; dd += df * df; }
              if (dd > best) { best = dd; loc = q; }
            }
            return loc;
          };
          if (mm > 0) pick[0] = farthest(0);
          if (meshdim > 1 && mm > 1) {
            pick[1] = farthest(pick[0]);
            if (pick[1] == pick[0])
              for (int q = 0; q < mm; ++q) if (q != pick[0]) { pick[1] = q; break; }
          }
          if (meshdim > 2 && mm > 2) {
            const double *p1 = &x[3 * pick[0]], *p2 = &x[3 * pick[1]];
            vector<double> area(mm);
            for (int q = 0; q < mm; ++q) {
              const double* pi = &x[3 * q];
              double t1 = (p2[1] - p1[1]) * (pi[2] - p1[2]) - (pi[1] - p1[1]) * (p2[2] - p1[2]);
              double t2 = (p2[0] - p1[0]) * (pi[2] - p1[2]) - (pi[0] - p1[0]) * (p2[2] - p1[2]);
              double t3 = (p2[0] - p1[0]) * (pi[1] - p1[1]) - (pi[0] - p1[0]) * (p2[1] - p1[1]);
              area[q] = t1 * t1 + t2 * t2 + t3 * t3;
            }
            double mv = 0.0;
            int ml = -1;
            for (int q = 0; q < mm; ++q) if (area[q] > mv) { mv = area[q]; ml = q; }
            pick[2] = ml;
            mv = 0.0; ml = -1;
            for (int q = mm - 1; q >= 0; --q) if (area[q] > mv) { mv = area[q]; ml = q; }
            pick[3] = ml;
            if ((pick[2] == pick[0] && pick[3] == pick[0]) || (pick[2] == pick[1] && pick[3] == pick[1])) {
              for (int q = 0; q < mm; ++q) if (q != pick[0] && q != pick[1]) { pick[2] = q; break; }
              for (int q = 0; q < mm; ++q) if (q != pick[0] && q != pick[1] && q != pick[2]) { pick[3] = q; break; }
            }
          }
          int nb = meshdim <= 2 ? 2 : 4;
          for (int k = 0; k < nb; ++k)
            if (pick[k] >= 0) type[shn[members[pick[k]]].second] = 3;
        }
      }
    }
    for (int i = 0; i < nnodi; ++i) if (type[i] == 3) pass1_corners[t].push_back(s.isngn[s.iin[i]]);
  }
  for (auto& v : pass1_corners)
    for (int g : v) corner_node[g] = 1;

  // ---- coarse numbering of a class of entities identified by a global node id:
  // owner = lowest subdomain index holding the node; numbers run over
  // subdomains in order, inside a subdomain in interface node order.
  // (arrays indexed by global node id: num 0 = not numbered)
  auto number_entities = [&](int shift, const vector<vector<int>>& ent_gid, vector<vector<int>>& ent_num) {
    // the entities each subdomain owns, in its interface node order; then
    // offsets over the subdomains, and the numbers
    vector<vector<int>> owned(nsub);
    vector<int> off(nsub + 1, 0);
#pragma omp parallel for schedule(dynamic)
    for (int t = 0; t < nsub; ++t) {
      auto& s = S.subs[t];
      static thread_local vector<char> mine;  // marks of t's entities, cleared after use
      if ((int)mine.size() < nnod_global) mine.assign(nnod_global, 0);
      for (int g : ent_gid[t]) mine[g] = 1;
      for (int i = 0; i < s.nnodi; ++i) {
        const int g = s.isngn[s.iin[i]];
        if (mine[g] && sh.sub[sh.ptr[g]] == t) owned[t].push_back(g);
      }
      for (int g : ent_gid[t]) mine[g] = 0;
      off[t + 1] = (int)owned[t].size();
    }
    for (int t = 0; t < nsub; ++t) off[t + 1] += off[t];
    vector<int> num(nnod_global, 0);
#pragma omp parallel for schedule(dynamic)
    for (int t = 0; t < nsub; ++t) {
      int next = shift + 1 + off[t];
      for (int g : owned[t]) num[g] = next++;
    }
    ent_num.resize(nsub);
    int orphan = 0;
#pragma omp parallel for schedule(dynamic) reduction(| : orphan)
    for (int t = 0; t < nsub; ++t) {
      ent_num[t].resize(ent_gid[t].size());
      for (size_t e = 0; e < ent_gid[t].size(); ++e) {
        const int n = num[ent_gid[t][e]];
        orphan |= n == 0;
        ent_num[t][e] = n;
      }
    }
    if (orphan) throw Error{ERR_NUMERIC, "coarse entity without owner"};
    return off[nsub];
  };

  // corners of each subdomain, ascending global id
  vector<vector<int>> corner_gid(nsub), corner_num;
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    for (int i = 0; i < s.nnodi; ++i)
      if (corner_node[s.isngn[s.iin[i]]]) corner_gid[t].push_back(s.isngn[s.iin[i]]);
    std::sort(corner_gid[t].begin(), corner_gid[t].end());
  }
  S.ncorner = number_entities(0, corner_gid, corner_num);

  // ---- pass 2: edges and faces, Dirichlet node removal
  vector<vector<vector<int>>> edges(nsub), faces(nsub);  // node lists (inodi)
  vector<vector<int>> edge_gid(nsub), face_gid(nsub), edge_num, face_num;
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    {
      // non-corner nodes shared by more than one other subdomain form edges,
      // the others faces; one glob per signature
      vector<int> en, fn;
      for (int i = 0; i < s.nnodi; ++i) {
        if (corner_node[s.isngn[s.iin[i]]]) continue;
        (sigt[t].size(i) > 1 ? en : fn).push_back(i);
      }
      edges[t] = group_by_signature(sigt[t], en);
      faces[t] = group_by_signature(sigt[t], fn);
      SigTable().e.swap(sigt[t].e);
    }
    if (s.bc_present) {  // remove_bc_nodes on the first level (module_levels.f90:2233-2237)
      auto strip = [&](vector<vector<int>>& globs) {
        vector<vector<int>> kept;
        for (auto& gl : globs) {
          vector<int> k2;
          for (int i : gl) {
            int nd = s.iin[i];
            bool fixed = false;
            for (int d = 0; d < s.nndf[nd]; ++d) if (s.ifix[s.kdof[nd] + d] > 0) fixed = true;
            if (!fixed) k2.push_back(i);
          }
          if (!k2.empty()) kept.push_back(k2);
        }
        globs.swap(kept);
      };
      strip(edges[t]);
      strip(faces[t]);
    }
    for (auto& gl : edges[t]) {
      int mn = INT32_MAX;
      for (int i : gl) mn = std::min(mn, s.isngn[s.iin[i]]);
      edge_gid[t].push_back(mn);
    }
    for (auto& gl : faces[t]) {
      int mn = INT32_MAX;
      for (int i : gl) mn = std::min(mn, s.isngn[s.iin[i]]);
      face_gid[t].push_back(mn);
    }
  }
  S.nedge = number_entities(S.ncorner, edge_gid, edge_num);
  S.nface = number_entities(S.ncorner + S.nedge, face_gid, face_num);

  // ---- coarse nodes and constraints
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    s.cnodes.clear();
    // interface node of each corner (corner_gid[t] is ascending)
    const vector<int>& cg = corner_gid[t];
    vector<int> corner_inodi(cg.size(), -1);
    for (int i = 0; i < s.nnodi; ++i) {
      const int g = s.isngn[s.iin[i]];
      auto it = std::lower_bound(cg.begin(), cg.end(), g);
      if (it != cg.end() && *it == g) corner_inodi[it - cg.begin()] = i;
    }
    auto add = [&](int itype, int num, const vector<int>& nodes, bool used) {
      CoarseNode cn;
      cn.itype = itype;
      cn.global_number = num;
      cn.inodi = nodes;
      int ncd = 0;
      for (int i : nodes) {
        int nd = s.iin[i];
        ncd = std::max(ncd, s.nndf[nd]);
        for (int d = 0; d < s.nndf[nd]; ++d) cn.idofi.push_back(s.kdofi[i] + d);
      }
      cn.ncdof = used ? (itype == 3 ? s.nndf[s.iin[nodes[0]]] : ncd) : 0;
      cn.used = used;
      s.cnodes.push_back(std::move(cn));
    };
    s.cnodes.reserve(corner_gid[t].size() + edges[t].size() + faces[t].size());
    for (size_t c = 0; c < corner_gid[t].size(); ++c)
      add(3, corner_num[t][c], {corner_inodi[c]}, S.prm.use_corner);
    for (size_t e = 0; e < edges[t].size(); ++e) add(2, edge_num[t][e], edges[t][e], S.prm.use_arith);
    for (size_t f = 0; f < faces[t].size(); ++f) add(1, face_num[t][f], faces[t][f], S.prm.use_arith);
  }
  host_constraint_rows(S);

  // ---- unique interface dofs (numbered in ascending global dof id) and per-dof sharing lists
  vector<int> gdof_uniq(ndof_global, -1);
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    const auto& s = S.subs[t];
    for (int i = 0; i < s.ndofi; ++i) {
      const int g = s.isvgvn[s.iivsvn[i]];
#pragma omp atomic write
      gdof_uniq[g] = -2;  // marks (several subdomains mark a shared dof)
    }
  }
  {  // marked dofs numbered in ascending global id: per-thread counts of contiguous id ranges, then offsets
    vector<int> cnt(omp_get_max_threads() + 1, 0);
    int nused = 1;
#pragma omp parallel num_threads((int)cnt.size() - 1)
    {
      const int nt = omp_get_num_threads(), th = omp_get_thread_num();
      const int g0 = (int)((long)ndof_global * th / nt), g1 = (int)((long)ndof_global * (th + 1) / nt);
      int c = 0;
      for (int g = g0; g < g1; ++g) c += gdof_uniq[g] == -2;
      cnt[th + 1] = c;
#pragma omp barrier
#pragma omp single
      {
        for (int q = 0; q < nt; ++q) cnt[q + 1] += cnt[q];
        nused = nt;
      }
      int nu = cnt[th];
      for (int g = g0; g < g1; ++g)
        if (gdof_uniq[g] == -2) gdof_uniq[g] = nu++;
    }
    S.ninterface = cnt[nused];
  }
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    s.uniq.resize(s.ndofi);
    for (int i = 0; i < s.ndofi; ++i) s.uniq[i] = gdof_uniq[s.isvgvn[s.iivsvn[i]]];
  }
  // owners of each unique dof, ascending subdomain
  vector<int> optr, osub, oloc;
  owner_lists(S, optr, osub, oloc);
  // own value plus the other holders' values in ascending order (the
  // upload / swap / download sum of module_dd.f90:11236-11551)
  auto neighbour_sum = [&](int t, int i, const std::function<double(int, int)>& val) {
    int u = S.subs[t].uniq[i];
    double own = val(t, i), acc = 0.0;
    for (int q = optr[u]; q < optr[u + 1]; ++q) if (osub[q] != t) acc += val(osub[q], oloc[q]);
    return std::make_pair(own, acc);
  };

  // ---- assembled Dirichlet contributions on the interface (module_dd.f90:1200-1255)
  host_interface_bc(S);

  // ---- weights (module_dd.f90:11554-11722)
  {
    vector<vector<double>> rho(nsub);
    for (int t = 0; t < nsub; ++t) {
      auto& s = S.subs[t];
      rho[t].assign(s.ndofi, 1.0);
      if (S.prm.weights_type == 1) {
        vector<double> dg(s.ndof, 0.0);
        for (size_t k = 0; k < s.ia.size(); ++k) if (s.ia[k] == s.ja[k]) dg[s.ia[k]] += s.a[k];
        for (int i = 0; i < s.ndofi; ++i) { rho[t][i] = dg[s.iivsvn[i]]; if (rho[t][i] == 0.0) rho[t][i] = 1.0; }
      } else if (S.prm.weights_type != 0) {
        throw Error{ERR_UNSUPPORTED, "weights_type " + std::to_string(S.prm.weights_type) + " is not implemented"};
      }
    }
    int zero_den = 0;  // an exception may not leave the parallel loop: flag, then throw
#pragma omp parallel for schedule(dynamic) reduction(| : zero_den)
    for (int t = 0; t < nsub; ++t) {
      auto& s = S.subs[t];
      s.wi.resize(s.ndofi);
      for (int i = 0; i < s.ndofi; ++i) {
        auto pr = neighbour_sum(t, i, [&](int a, int b) { return rho[a][b]; });
        double den = pr.first + pr.second;
        zero_den |= den == 0.0;
        s.wi[i] = den == 0.0 ? 0.0 : pr.first / den;
      }
      s.rhoi = rho[t];
    }
    if (zero_den) throw Error{ERR_NUMERIC, "zero denominator in interface weights"};
  }
  S.iface_fixed.assign(S.ninterface, 0);
  S.iface_wsum.assign(S.ninterface, 0.0);
  for (auto& s : S.subs)
    for (int i = 0; i < s.ndofi; ++i) {
      if (s.ifix[s.iivsvn[i]]) S.iface_fixed[s.uniq[i]] = 1;
      S.iface_wsum[s.uniq[i]] += s.wi[i];
    }

  S.stats.ncorner = S.ncorner; S.stats.nedge = S.nedge; S.stats.nface = S.nface; S.stats.ndofc = S.ndofc;
  S.stats.sum_ndofi = 0; S.stats.sum_ndofo = 0;
  for (auto& s : S.subs) { S.stats.sum_ndofi += s.ndofi; S.stats.sum_ndofo += s.ndofo; }
  S.stats.ninterface = S.ninterface;
  S.ndof_global = ndof_global;
  S.stats.t_host_globs = wall_time() - tt;
  // ---- device-ready blocks (interior reordering, CSR splits, reduced-rhs inputs)
  tt = wall_time();
  S.blocks.assign(nsub, SubBlocks{});
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) host_prepare_blocks(S.subs[t], S.blocks[t]);
  S.stats.t_host_blocks = wall_time() - tt;
  S.stats.band_w = 0;
  for (auto& b : S.blocks) S.stats.band_w = std::max(S.stats.band_w, (double)b.w);
}

// ---------------------------------------------------- device-ready blocks

// reduced-rhs input: weighted rhs, Dirichlet rows zeroed, weighted bc added
// (module_dd.f90:7040-7075 and sm_prepare_rhs, module_sm.f90:603-628)
void host_reduced_rhs_inputs(const Subdomain& s, vector<double>& fo, vector<double>& fi) {
  host_reduced_rhs_inputs(s, s.rhs.data(), s.rhs_complete, fo, fi);
}

void host_reduced_rhs_inputs(const Subdomain& s, const double* rhs, bool complete, vector<double>& fo,
                             vector<double>& fi) {
  const int no = s.ndofo, ni = s.ndofi;
  vector<double> f(rhs, rhs + s.ndof);
  vector<double> bcw = s.bc;
  if (complete) for (int i = 0; i < ni; ++i) f[s.iivsvn[i]] *= s.wi[i];
  for (int i = 0; i < ni; ++i) bcw[s.iivsvn[i]] *= s.wi[i];
  if (s.bc_present)
    for (int i = 0; i < s.ndof; ++i) { if (s.ifix[i]) f[i] = 0.0; f[i] += bcw[i]; }
  fo.resize(no);
  for (int q = 0; q < no; ++q) fo[q] = f[s.iovsvn[s.operm[q]]];
  fi.resize(ni);
  for (int i = 0; i < ni; ++i) fi[i] = f[s.iivsvn[i]];
}

void host_prepare_blocks(Subdomain& s, SubBlocks& b) {
  constexpr int NB = 64;
  // the full matrix is scratch: one set of buffers per thread, reused across subdomains
  static thread_local vector<int> fptr, fcol;
  static thread_local vector<double> fval;
  full_symmetric_csr(s, fptr, fcol, fval);
  host_interior_ordering(s, fptr, fcol, fval);
  int no = s.ndofo, ni = s.ndofi;
  vector<int> onew(s.ndof, -1), iidx(s.ndof, -1);
  for (int q = 0; q < no; ++q) onew[s.iovsvn[s.operm[q]]] = q;
  for (int i = 0; i < ni; ++i) iidx[s.iivsvn[i]] = i;
  // the rows of one dof set (interior rows in the band order, or interface
  // rows) split by column into the interior block and the interface block in
  // one pass; each block keeps the row's column order.  Explicit zeros (the
  // removed couplings of fixed dofs) are left out, so that they do not widen
  // the band; diagonal entries are always kept.
  struct Out {
    vector<int>* ptr;
    rawvec<int>* col;
    rawvec<double>* val;
    int* maxrow;
  };
  auto build = [&](int nrow, auto rowdof, Out o, Out i) {
    o.ptr->assign(nrow + 1, 0);
    i.ptr->assign(nrow + 1, 0);
    *o.maxrow = 0;
    *i.maxrow = 0;
    for (int r = 0; r < nrow; ++r) {
      int d = rowdof(r), co = 0, ci = 0;
      for (int k = fptr[d]; k < fptr[d + 1]; ++k) {
        const int c = fcol[k];
        if (fval[k] != 0.0 || c == d) {
          co += onew[c] >= 0;
          ci += iidx[c] >= 0;
        }
      }
      (*o.ptr)[r + 1] = (*o.ptr)[r] + co;
      (*i.ptr)[r + 1] = (*i.ptr)[r] + ci;
      *o.maxrow = std::max(*o.maxrow, co);
      *i.maxrow = std::max(*i.maxrow, ci);
    }
    o.col->resize((*o.ptr)[nrow]);
    o.val->resize((*o.ptr)[nrow]);
    i.col->resize((*i.ptr)[nrow]);
    i.val->resize((*i.ptr)[nrow]);
    int* oc = o.col->data();
    int* ic = i.col->data();
    double* ov = o.val->data();
    double* iv = i.val->data();
    for (int r = 0; r < nrow; ++r) {
      int d = rowdof(r), qo = (*o.ptr)[r], qi = (*i.ptr)[r];
      for (int k = fptr[d]; k < fptr[d + 1]; ++k) {
        const int c = fcol[k];
        if (fval[k] != 0.0 || c == d) {
          if (onew[c] >= 0) { oc[qo] = onew[c]; ov[qo++] = fval[k]; }
          if (iidx[c] >= 0) { ic[qi] = iidx[c]; iv[qi++] = fval[k]; }
        }
      }
    }
  };
  auto orow = [&](int r) { return s.iovsvn[s.operm[r]]; };
  auto irow = [&](int r) { return s.iivsvn[r]; };
  build(no, orow, Out{&b.oo_ptr, &b.oo_col, &b.oo_val, &b.maxrow_oo},
        Out{&b.oi_ptr, &b.oi_col, &b.oi_val, &b.maxrow_oi});
  build(ni, irow, Out{&b.io_ptr, &b.io_col, &b.io_val, &b.maxrow_io},
        Out{&b.ii_ptr, &b.ii_col, &b.ii_val, &b.maxrow_ii});
  b.w = 0;
  for (int r = 0; r < no; ++r)
    for (int k = b.oo_ptr[r]; k < b.oo_ptr[r + 1]; ++k)
      if (b.oo_col[k] <= r) b.w = std::max(b.w, r / NB - b.oo_col[k] / NB);
  host_reduced_rhs_inputs(s, b.fo, b.fi);
  double sd = 0.0;
  int cnt = 0;
  for (int i = 0; i < ni; ++i)
    for (int k = b.ii_ptr[i]; k < b.ii_ptr[i + 1]; ++k)
      if (b.ii_col[k] == i) { sd += std::fabs(b.ii_val[k]); cnt++; }
  b.rho = cnt ? sd / cnt : 1.0;
  if (!(b.rho > 0.0)) b.rho = 1.0;
}


}  // namespace bddc
