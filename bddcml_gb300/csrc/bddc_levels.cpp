// Three-level BDDC, host part: the level-2 problem built from the level-1
// coarse space (levels_prepare_standard_level, module_levels.f90:1297-3000).
//
// Level 2 is a mesh whose nodes are the level-1 coarse nodes (corners, edges,
// faces; coordinates = the node, or the mean of the glob's nodes,
// module_dd.f90:4946-4994), whose elements are the level-1 subdomains (element
// matrix = the subdomain's local coarse matrix Phi^T S Phi, dd_get_coarsem /
// dd_gather_matrix), divided into the level-2 subdomains.  The reference
// divides with METIS; here the division is a recursive coordinate bisection
// of the level-1 subdomain centroids (longest extent first, halves by count).
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <memory>
#include <numeric>
#include <string>

#include "bddc_internal.hpp"

namespace bddc {

Solver::~Solver() {
  lev2.reset();  // the level-2 device state goes first: it uses this level's stream
  if (dev) device_destroy(dev);
}

namespace {

void bisect(vector<int> ids, int nparts, int first, const vector<std::array<double, 3>>& c, int ndim,
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
  std::sort(ids.begin(), ids.end(), [&](int x, int y) {
    return c[x][axis] != c[y][axis] ? c[x][axis] < c[y][axis] : x < y;
  });
  const int k1 = nparts / 2;
  const size_t n1 = ids.size() * (size_t)k1 / (size_t)nparts;
  vector<int> a(ids.begin(), ids.begin() + n1), b(ids.begin() + n1, ids.end());
  bisect(a, k1, first, c, ndim, part);
  bisect(b, nparts - k1, first + k1, c, ndim, part);
}

}  // namespace

vector<int> host_level_division(const vector<std::array<double, 3>>& centroids, int ndim, int nparts) {
  vector<int> part(centroids.size(), 0), ids(centroids.size());
  std::iota(ids.begin(), ids.end(), 0);
  bisect(ids, nparts, 0, centroids, ndim, part);
  return part;
}

std::unique_ptr<Solver> host_build_level2(const Solver& S1, const vector<vector<double>>& acs, int nsub2) {
  const int nsub1 = (int)S1.subs.size();
  const int ndim = S1.subs.empty() ? 3 : S1.subs[0].ndim;
  const int ncnode = S1.ncorner + S1.nedge + S1.nface;
  // coarse nodes: dofs, first global coarse dof, coordinates
  vector<int> ncd(ncnode, 0), kdc(ncnode, -1);
  vector<std::array<double, 3>> xc(ncnode, {0.0, 0.0, 0.0});
  vector<std::array<double, 3>> cent(nsub1, {0.0, 0.0, 0.0});
  for (int t = 0; t < nsub1; ++t) {
    const Subdomain& s = S1.subs[t];
    for (int i = 0; i < s.nnod; ++i)
      for (int d = 0; d < ndim; ++d) cent[t][d] += s.xyz[(size_t)d * s.nnod + i] / s.nnod;
    int r = 0;
    for (const CoarseNode& cn : s.cnodes) {
      if (!cn.used) continue;
      const int g = cn.global_number - 1;
      if (kdc[g] < 0) {
        ncd[g] = cn.ncdof;
        kdc[g] = s.indrowc[r];
        for (int i : cn.inodi) {
          const int nd = s.iin[i];
          for (int d = 0; d < ndim; ++d) xc[g][d] += s.xyz[(size_t)d * s.nnod + nd] / (double)cn.inodi.size();
        }
      }
      r += cn.ncdof;
    }
  }
  vector<int> part = host_level_division(cent, ndim, nsub2);
  auto S2 = std::make_unique<Solver>();
  S2->prm = S1.prm;
  S2->prm.nlevels = 2;
  S2->prm.nsub = nsub2;
  S2->prm.numbase = 0;
  S2->prm.precision = 0;  // the small intermediate problem in FP64
  S2->prm.use_adaptive = false;
  S2->prm.matrixtype = 1;
  S2->subs.resize(nsub2);
  S2->nelem = nsub1;
  S2->nnod = ncnode;
  for (int t2 = 0; t2 < nsub2; ++t2) {
    Subdomain& q = S2->subs[t2];
    vector<int> elems;
    for (int t = 0; t < nsub1; ++t)
      if (part[t] == t2) elems.push_back(t);
    if (elems.empty()) throw Error{ERR_ARGUMENT, "an empty level-2 subdomain"};
    // nodes: the used coarse nodes of its elements, by global number
    std::map<int, int> loc;
    for (int t : elems)
      for (const CoarseNode& cn : S1.subs[t].cnodes)
        if (cn.used) loc.emplace(cn.global_number - 1, 0);
    int nn = 0, nd = 0;
    vector<int> kd;
    for (auto& kv : loc) {
      kv.second = nn++;
      q.isngn.push_back(kv.first);
      q.nndf.push_back(ncd[kv.first]);
      kd.push_back(nd);
      nd += ncd[kv.first];
    }
    q.nnod = nn;
    q.ndof = nd;
    q.ndim = ndim;
    q.nelem = (int)elems.size();
    q.isvgvn.resize(nd);
    q.xyz.assign((size_t)nn * ndim, 0.0);
    for (auto& kv : loc) {
      const int l = kv.second;
      for (int d = 0; d < ncd[kv.first]; ++d) q.isvgvn[kd[l] + d] = kdc[kv.first] + d;
      for (int d = 0; d < ndim; ++d) q.xyz[(size_t)d * nn + l] = xc[kv.first][d];
    }
    for (int t : elems) {
      const Subdomain& s = S1.subs[t];
      q.isegn.push_back(t);
      vector<int> rowdof;  // local level-2 dof of each row of the element matrix
      int cnt = 0;
      for (const CoarseNode& cn : s.cnodes) {
        if (!cn.used) continue;
        const int l = loc.at(cn.global_number - 1);
        q.inet.push_back(l);
        ++cnt;
        for (int d = 0; d < cn.ncdof; ++d) rowdof.push_back(kd[l] + d);
      }
      q.nnet.push_back(cnt);
      const int nc = (int)rowdof.size();
      const vector<double>& a = acs[t];
      for (int r = 0; r < nc; ++r)
        for (int c = 0; c < nc; ++c) {
          const int i = rowdof[r], j = rowdof[c];
          if (i < j || r == c) {
            q.ia.push_back(i);
            q.ja.push_back(j);
            q.a.push_back(r == c ? a[(size_t)r * nc + r] : 0.5 * (a[(size_t)r * nc + c] + a[(size_t)c * nc + r]));
          }
        }
    }
    q.ifix.assign(nd, 0);
    q.fixv.assign(nd, 0.0);
    q.rhs.assign(nd, 0.0);
    q.sol.assign(nd, 0.0);
    q.rhs_complete = true;
    q.matrixtype = 1;
    q.loaded = true;
    q.assembled = false;
    q.find_components = true;
    q.dual_graph = true;
    q.neighbouring = 1;
  }
  return S2;
}

}  // namespace bddc
