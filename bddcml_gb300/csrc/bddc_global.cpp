// Global loading: the mesh and data of the whole problem uploaded at once
// (levels_upload_global_data, module_levels.f90:422-612) and divided into the
// subdomains at setup.  The reference divides the element graph with METIS
// (module_levels.f90:1540-1560); here the elements are divided by a recursive
// coordinate bisection of their centroids into nsublev[0] parts, the division
// used for the level-2 problem as well.  Each subdomain then gets its elements
// in ascending global order, its nodes in ascending global order, the
// restrictions of the fixed values, loads (complete) and initial guess, and the
// element matrices read from the ELM file: one Fortran unformatted sequential
// record per element, "lelm, elm(1:lelm)" (dd_read_matrix_by_root,
// module_dd.f90:1015-1060), packed as sm_pmd_make_element_numbering does
// (module_sm.f90:272-380): for column jve of the element's dofs, rows ive = 1..jve
// (symmetric storage, entries below the diagonal mirrored) or 1..nve (general).
#include <algorithm>
#include <array>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "bddc_internal.hpp"

namespace bddc {

namespace {

// one record of a Fortran unformatted sequential file written with 4-byte
// record markers (gfortran's default): the payload length before and after.
// A payload longer than max_bytes is refused before anything is allocated.
bool read_record(std::FILE* f, vector<unsigned char>& buf, size_t max_bytes) {
  unsigned char m[4];
  if (std::fread(m, 1, 4, f) != 4) return false;
  uint32_t n;
  std::memcpy(&n, m, 4);
  if (n > max_bytes) return false;
  buf.resize(n);
  if (n && std::fread(buf.data(), 1, n, f) != n) return false;
  if (std::fread(m, 1, 4, f) != 4) return false;
  uint32_t n2;
  std::memcpy(&n2, m, 4);
  return n2 == n;
}

}  // namespace

void host_localize_global(Solver& S, int matrixtype) {
  GlobalData& G = S.global;
  const int nsub = (int)S.subs.size();
  if (nsub > G.nelem) throw Error{ERR_ARGUMENT, "more subdomains than elements"};
  vector<int> kinet(G.nelem + 1, 0);
  for (int e = 0; e < G.nelem; ++e) kinet[e + 1] = kinet[e] + G.nnet[e];
  vector<int> kdof(G.nnod + 1, 0);
  for (int n = 0; n < G.nnod; ++n) kdof[n + 1] = kdof[n] + G.nndf[n];
  // element division
  vector<std::array<double, 3>> cent(G.nelem, {0.0, 0.0, 0.0});
  for (int e = 0; e < G.nelem; ++e)
    for (int k = kinet[e]; k < kinet[e + 1]; ++k)
      for (int d = 0; d < G.ndim; ++d) cent[e][d] += G.xyz[(size_t)d * G.nnod + G.inet[k]] / G.nnet[e];
  vector<int> part = host_level_division(cent, G.ndim, nsub);
  // local numbering
  vector<vector<int>> elems(nsub);
  for (int e = 0; e < G.nelem; ++e) elems[part[e]].push_back(e);
  vector<int> lnode(G.nnod, -1);
  for (int t = 0; t < nsub; ++t) {
    Subdomain& s = S.subs[t];
    if (elems[t].empty()) throw Error{ERR_ARGUMENT, "an empty subdomain after the element division"};
    vector<int> nodes;
    for (int e : elems[t])
      for (int k = kinet[e]; k < kinet[e + 1]; ++k) nodes.push_back(G.inet[k]);
    std::sort(nodes.begin(), nodes.end());
    nodes.erase(std::unique(nodes.begin(), nodes.end()), nodes.end());
    s = Subdomain{};
    s.nelem = (int)elems[t].size();
    s.nnod = (int)nodes.size();
    s.ndim = G.ndim;
    s.isngn = nodes;
    s.isegn = elems[t];
    s.nndf.resize(s.nnod);
    s.xyz.assign((size_t)s.nnod * G.ndim, 0.0);
    for (int i = 0; i < s.nnod; ++i) {
      const int g = nodes[i];
      s.nndf[i] = G.nndf[g];
      for (int d = 0; d < G.ndim; ++d) s.xyz[(size_t)d * s.nnod + i] = G.xyz[(size_t)d * G.nnod + g];
      for (int q = kdof[g]; q < kdof[g + 1]; ++q) s.isvgvn.push_back(q);
    }
    s.ndof = (int)s.isvgvn.size();
    for (int i = 0; i < s.nnod; ++i) lnode[nodes[i]] = i;
    for (int e : elems[t]) {
      s.nnet.push_back(G.nnet[e]);
      for (int k = kinet[e]; k < kinet[e + 1]; ++k) s.inet.push_back(lnode[G.inet[k]]);
    }
    for (int i = 0; i < s.nnod; ++i) lnode[nodes[i]] = -1;
    s.ifix.resize(s.ndof);
    s.fixv.resize(s.ndof);
    s.rhs.resize(s.ndof);
    s.sol.resize(s.ndof);
    for (int q = 0; q < s.ndof; ++q) {
      const int g = s.isvgvn[q];
      s.ifix[q] = G.ifix[g];
      s.fixv[q] = G.fixv[g];
      s.rhs[q] = G.rhs[g];
      s.sol[q] = G.sol[g];
    }
    s.rhs_complete = true;
    s.matrixtype = matrixtype;
    s.assembled = false;
    s.find_components = true;
    s.dual_graph = true;
    s.neighbouring = G.neighbouring;
  }
  // element matrices, read in global element order
  std::FILE* f = std::fopen(G.elm_file.c_str(), "rb");
  if (!f) throw Error{ERR_ARGUMENT, "cannot open the element matrix file " + G.elm_file};
  std::unique_ptr<std::FILE, int (*)(std::FILE*)> guard(f, &std::fclose);
  vector<int> lpos(G.ndof, -1);  // global dof -> local dof of the element's subdomain
  vector<unsigned char> rec;
  vector<int> kdofe;
  for (int e = 0; e < G.nelem; ++e) {
    Subdomain& s = S.subs[part[e]];
    kdofe.clear();
    for (int k = kinet[e]; k < kinet[e + 1]; ++k)
      for (int q = kdof[G.inet[k]]; q < kdof[G.inet[k] + 1]; ++q) kdofe.push_back(q);
    const int nve = (int)kdofe.size();
    const long long lelm_expected = matrixtype == 0 ? (long long)nve * nve : (long long)nve * (nve + 1) / 2;
    if (!read_record(f, rec, 4 + 8 * (size_t)lelm_expected))
      throw Error{ERR_ARGUMENT, "element matrix file ends early or is damaged"};
    int lelm = 0;
    if (rec.size() >= 4) std::memcpy(&lelm, rec.data(), 4);
    if (lelm != lelm_expected || rec.size() != 4 + 8 * (size_t)lelm)
      throw Error{ERR_ARGUMENT, "element " + std::to_string(e + 1) + ": record length does not match its dofs"};
    // global dof -> subdomain-local dof for this element's dofs
    for (int q = 0; q < nve; ++q) {
      const int g = kdofe[q];
      lpos[g] = (int)(std::lower_bound(s.isvgvn.begin(), s.isvgvn.end(), g) - s.isvgvn.begin());
    }
    const unsigned char* v = rec.data() + 4;
    int inda = 0;
    for (int jve = 0; jve < nve; ++jve) {
      const int ub = matrixtype == 0 ? nve : jve + 1;
      for (int ive = 0; ive < ub; ++ive, ++inda) {
        double a;
        std::memcpy(&a, v + 8 * (size_t)inda, 8);
        int i = lpos[kdofe[ive]], j = lpos[kdofe[jve]];
        if (matrixtype != 0 && i > j) std::swap(i, j);
        s.ia.push_back(i);
        s.ja.push_back(j);
        s.a.push_back(a);
      }
    }
  }
  for (auto& s : S.subs) s.loaded = true;
  S.nelem = G.nelem;
  S.nnod = G.nnod;
}

}  // namespace bddc
