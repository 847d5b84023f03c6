// C ABI of the GB300 BDDC solver: the bddcml_*_c entry points of the
// reference header src/bddcml_interface_c.h with identical signatures, over
// one global solver instance (the reference keeps its state in module
// variables, module_levels.f90:158-175, module_krylov.f90:33-43).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

#include "../../include/bddcml_gb300.h"
#include "bddc_internal.hpp"

using namespace bddc;

namespace {

std::unique_ptr<Solver> g_solver;
int g_status = BDDCML_OK;
std::string g_msg;

void set_error(int code, const std::string& msg) {
  g_status = code;
  g_msg = msg;
}

void clear_error() {
  g_status = BDDCML_OK;
  g_msg.clear();
}

Solver* need_solver(const char* who) {
  if (!g_solver) {
    set_error(BDDCML_ERR_ARGUMENT, std::string(who) + ": bddcml_init_c has not been called");
    return nullptr;
  }
  return g_solver.get();
}

template <typename F>
void guarded(const char* who, F&& f) {
  clear_error();
  try {
    f();
  } catch (Error& e) {
    set_error(e.code, std::string(who) + ": " + e.msg);
  } catch (std::bad_alloc&) {
    set_error(BDDCML_ERR_MEMORY, std::string(who) + ": host allocation failed");
  } catch (std::exception& e) {
    set_error(BDDCML_ERR_ARGUMENT, std::string(who) + ": " + e.what());
  }
}

int sub_index(Solver& S, int isub_in) {
  int t = isub_in - S.prm.numbase;
  if (t < 0 || t >= (int)S.subs.size())
    throw Error{ERR_ARGUMENT, "subdomain index " + std::to_string(isub_in) + " out of range"};
  return t;
}

}  // namespace

extern "C" {

void bddcml_init_c(int* nl, int* nsublev, int* lnsublev, int* nsub_loc_1, int* comm_init, int* verbose_level,
                   int* numbase, int* just_direct_solve_int) {
  guarded("bddcml_init_c", [&] {
    (void)comm_init;
    if (!nl || !nsublev || !lnsublev || !nsub_loc_1 || !numbase)
      throw Error{ERR_ARGUMENT, "null argument"};
    if (*nl < 2) throw Error{ERR_ARGUMENT, "number of levels must be at least 2"};
    if (*lnsublev < *nl) throw Error{ERR_ARGUMENT, "lnsublev smaller than the number of levels"};
    if (nsublev[*nl - 1] != 1) throw Error{ERR_ARGUMENT, "number of subdomains at the last level must be 1"};
    if (*nl > 3 || *nl < 2) throw Error{ERR_UNSUPPORTED, "2 or 3 levels are implemented"};
    if (*nl == 3 && (nsublev[1] < 1 || nsublev[1] > nsublev[0]))
      throw Error{ERR_ARGUMENT, "level-2 subdomain count must be between 1 and the level-1 count"};
    if (just_direct_solve_int && *just_direct_solve_int)
      throw Error{ERR_UNSUPPORTED, "the global direct solve (just_direct_solve) is not implemented"};
    if (*nsub_loc_1 != -1 && *nsub_loc_1 != nsublev[0])
      throw Error{ERR_ARGUMENT, "all subdomains live in this process: nsub_loc_1 must be -1 or nsublev[0]"};
    g_solver.reset();  // the solver destroys its device state
    auto S = std::make_unique<Solver>();
    S->prm.nlevels = *nl;
    S->prm.nsub = nsublev[0];
    S->prm.nsub2 = *nl == 3 ? nsublev[1] : 1;
    S->prm.numbase = *numbase;
    S->prm.verbose = verbose_level ? *verbose_level : 0;
    S->subs.resize(nsublev[0]);
    *nsub_loc_1 = nsublev[0];
    g_solver = std::move(S);
  });
}

void bddcml_upload_global_data_c(int*, int*, int*, int*, int*, int*, int*, int*, int*, int*, int*, double*, int*,
                                 int*, int*, int*, double*, int*, double*, int*, double*, int*, int*, int*, int*) {
  clear_error();
  set_error(BDDCML_ERR_UNSUPPORTED, "bddcml_upload_global_data_c: global data loading is not implemented");
}

void bddcml_upload_global_data_file_c(int* nelem, int* nnod, int* ndof, int* ndim, int* meshdim, int* inet,
                                      int* linet, int* nnet, int* lnnet, int* nndf, int* lnndf, double* xyz,
                                      int* lxyz1, int* lxyz2, int* ifix, int* lifix, double* fixv, int* lfixv,
                                      double* rhs, int* lrhs, double* sol, int* lsol, const char* elm_file,
                                      int* neighbouring, int* load_division_int) {
  guarded("bddcml_upload_global_data_file_c", [&] {
    Solver* S = need_solver("bddcml_upload_global_data_file_c");
    if (!S) return;
    if (load_division_int && *load_division_int)
      throw Error{ERR_UNSUPPORTED, "loading a stored element division is not implemented"};
    if (!elm_file) throw Error{ERR_ARGUMENT, "no element matrix file"};
    for (auto& s : S->subs)
      if (s.loaded) throw Error{ERR_ARGUMENT, "subdomain data were uploaded already"};
    if (*lnnet != *nelem || *lnndf != *nnod || *lxyz1 != *nnod || *lxyz2 != *ndim || *lifix != *ndof ||
        *lfixv != *ndof || *lrhs != *ndof || *lsol != *ndof)
      throw Error{ERR_ARGUMENT, "array length does not match nelem/nnod/ndof/ndim"};
    long long snn = 0, snd = 0;
    for (int e = 0; e < *nelem; ++e) snn += nnet[e];
    for (int n = 0; n < *nnod; ++n) snd += nndf[n];
    if (snn != *linet) throw Error{ERR_ARGUMENT, "NNET does not sum up to LINET"};
    if (snd != *ndof) throw Error{ERR_ARGUMENT, "NNDF does not sum up to NDOF"};
    GlobalData& G = S->global;
    G = GlobalData{};
    G.nelem = *nelem; G.nnod = *nnod; G.ndof = *ndof; G.ndim = *ndim; G.meshdim = *meshdim;
    G.neighbouring = neighbouring ? *neighbouring : 1;
    const int nb = S->prm.numbase;
    G.inet.resize(*linet);
    for (int k = 0; k < *linet; ++k) {
      G.inet[k] = inet[k] - nb;
      if (G.inet[k] < 0 || G.inet[k] >= *nnod) throw Error{ERR_ARGUMENT, "INET entry out of range"};
    }
    G.nnet.assign(nnet, nnet + *nelem);
    G.nndf.assign(nndf, nndf + *nnod);
    G.xyz.assign(xyz, xyz + (size_t)(*nnod) * (*ndim));
    G.ifix.assign(ifix, ifix + *ndof);
    G.fixv.assign(fixv, fixv + *ndof);
    G.rhs.assign(rhs, rhs + *ndof);
    G.sol.assign(sol, sol + *ndof);
    G.elm_file = elm_file;
    G.present = true;
    S->setup_done = false;
  });
}

void bddcml_upload_subdomain_data_c(int* nelem, int* nnod, int* ndof, int* ndim, int* meshdim, int* isub,
                                    int* nelems, int* nnods, int* ndofs, int* inet, int* linet, int* nnet,
                                    int* lnnet, int* nndf, int* lnndf, int* isngn, int* lisngn, int* isvgvn,
                                    int* lisvgvn, int* isegn, int* lisegn, double* xyz, int* lxyz1, int* lxyz2,
                                    int* ifix, int* lifix, double* fixv, int* lfixv, double* rhs, int* lrhs,
                                    int* is_rhs_complete, double* sol, int* lsol, int* matrixtype, int* i_sparse,
                                    int* j_sparse, double* a_sparse, int* la, int* is_assembled_int,
                                    double* user_constraints, int* luser_constraints1, int* luser_constraints2,
                                    double* element_data, int* lelement_data1, int* lelement_data2,
                                    double* dof_data, int* ldof_data, int* find_components_int,
                                    int* use_dual_mesh_graph_int, int* neighbouring) {
  double tup = wall_time();
  guarded("bddcml_upload_subdomain_data_c", [&] {
    Solver* S = need_solver("bddcml_upload_subdomain_data_c");
    if (!S) return;
    (void)user_constraints; (void)element_data; (void)dof_data; (void)meshdim;
    (void)luser_constraints2; (void)lelement_data1; (void)lelement_data2; (void)ldof_data;
    if (luser_constraints1 && *luser_constraints1 > 0)
      throw Error{ERR_UNSUPPORTED, "user constraints are not implemented"};
    int t = sub_index(*S, *isub);
    Subdomain& s = S->subs[t];
    if (s.loaded) throw Error{ERR_ARGUMENT, "mesh already loaded for this subdomain"};
    const int nb = S->prm.numbase;
    if (*lnnet != *nelems || *lnndf != *nnods || *lisngn != *nnods || *lisegn != *nelems || *lxyz1 != *nnods ||
        *lxyz2 != *ndim || *lisvgvn != *ndofs || *lifix != *ndofs || *lfixv != *ndofs || *lrhs != *ndofs ||
        *lsol != *ndofs)
      throw Error{ERR_ARGUMENT, "array length does not match nelems/nnods/ndofs/ndim"};
    // the sizes are copied to locals: the loops below store ints, which the
    // compiler would otherwise have to assume may overwrite *nelems and friends
    const int ne = *nelems, nn = *nnods, nd = *ndofs, nin = *linet;
    long sum_nnet = 0;
    for (int e = 0; e < ne; ++e) {
      if (nnet[e] < 0) throw Error{ERR_ARGUMENT, "negative NNET entry"};
      sum_nnet += nnet[e];
    }
    if (sum_nnet != nin) throw Error{ERR_ARGUMENT, "NNET does not sum up to LINET"};
    long sum_nndf = 0;
    for (int i = 0; i < nn; ++i) {
      if (nndf[i] < 0) throw Error{ERR_ARGUMENT, "negative NNDF entry"};
      sum_nndf += nndf[i];
    }
    if (sum_nndf != nd) throw Error{ERR_ARGUMENT, "NNDF does not sum up to NDOFS"};
    s.nelem = ne; s.nnod = nn; s.ndof = nd; s.ndim = *ndim;
    if (*matrixtype < 0 || *matrixtype > 2)
      throw Error{ERR_ARGUMENT, "matrixtype must be 0 (general), 1 (SPD) or 2 (symmetric)"};
    s.matrixtype = *matrixtype;
    s.rhs_complete = is_rhs_complete && *is_rhs_complete != 0;
    // Every array is copied in one parallel region, each loop split over the
    // threads: the triplets are most of the bytes, and the mesh arrays of a
    // large subdomain are too many for one thread's share of the memory
    // bandwidth.  Index arrays are shifted to 0-based and checked: local node
    // numbers must index the subdomain's nodes, global numbers (which index
    // tables over all subdomains) must not be negative.
    const int nla = *la;
    const long nxyz = (long)nn * (*ndim);
    s.inet.resize(nin); s.nnet.resize(ne); s.nndf.resize(nn);
    s.isngn.resize(nn); s.isvgvn.resize(nd); s.isegn.resize(ne);
    s.xyz.resize(nxyz); s.ifix.resize(nd); s.fixv.resize(nd); s.rhs.resize(nd); s.sol.resize(nd);
    s.ia.resize(nla); s.ja.resize(nla); s.a.resize(nla);
    int* pinet = s.inet.data();
    int* pnnet = s.nnet.data();
    int* pnndf = s.nndf.data();
    int* pisngn = s.isngn.data();
    int* pisvgvn = s.isvgvn.data();
    int* pisegn = s.isegn.data();
    int* pifix = s.ifix.data();
    double* pxyz = s.xyz.data();
    double* pfixv = s.fixv.data();
    double* prhs = s.rhs.data();
    double* psol = s.sol.data();
    int* ia = s.ia.data();
    int* ja = s.ja.data();
    double* av = s.a.data();
    int bad_index = 0, bad_order = 0, bad_range = 0;
#pragma omp parallel reduction(| : bad_index, bad_order, bad_range) if (nla > 65536)
    {
#pragma omp for schedule(static) nowait
      for (int k = 0; k < nin; ++k) {
        const int v = inet[k] - nb;
        pinet[k] = v;
        bad_index |= (v < 0) | (v >= nn);
      }
#pragma omp for schedule(static) nowait
      for (int i = 0; i < nn; ++i) {
        const int v = isngn[i] - nb;
        pisngn[i] = v;
        pnndf[i] = nndf[i];
        bad_index |= v < 0;
      }
#pragma omp for schedule(static) nowait
      for (int i = 0; i < nd; ++i) {
        const int v = isvgvn[i] - nb;
        pisvgvn[i] = v;
        bad_index |= v < 0;
        pifix[i] = ifix[i];
        pfixv[i] = fixv[i];
        prhs[i] = rhs[i];
        psol[i] = sol[i];
      }
#pragma omp for schedule(static) nowait
      for (int e = 0; e < ne; ++e) {
        const int v = isegn[e] - nb;
        pisegn[e] = v;
        pnnet[e] = nnet[e];
        bad_index |= v < 0;
      }
#pragma omp for schedule(static) nowait
      for (long k = 0; k < nxyz; ++k) pxyz[k] = xyz[k];
#pragma omp for schedule(static) nowait
      for (int k = 0; k < nla; ++k) {
        const int i = i_sparse[k] - nb, j = j_sparse[k] - nb;
        ia[k] = i;
        ja[k] = j;
        av[k] = a_sparse[k];
        bad_order |= i > j;
        bad_range |= (i < 0) | (i >= nd) | (j < 0) | (j >= nd);  // both bounds: general storage has i > j
      }
    }
    if (bad_index)
      throw Error{ERR_ARGUMENT, "INET entry outside the subdomain's nodes, or a negative global index"};
    if (bad_order && *matrixtype != 0)  // module_levels.f90:748-752
      throw Error{ERR_ARGUMENT, "matrix in wrong format - only the upper triangle is expected for symmetric problems"};
    if (bad_range) throw Error{ERR_ARGUMENT, "matrix index out of range"};
    // assembly (merge of repeated entries) and mesh components are computed
    // for all subdomains in parallel at setup
    s.assembled = false;
    (void)is_assembled_int;
    s.find_components = find_components_int && *find_components_int != 0;
    s.dual_graph = use_dual_mesh_graph_int && *use_dual_mesh_graph_int != 0;
    s.neighbouring = neighbouring ? *neighbouring : 1;
    s.loaded = true;
    (void)nelem; (void)nnod; (void)ndof;
    S->nelem = *nelem; S->nnod = *nnod;
    S->setup_done = false;
    S->t_upload += wall_time() - tup;
  });
}

void bddcml_setup_preconditioner_c(int* matrixtype, int* use_defaults_int, int* parallel_division_int,
                                   int* use_corner_constraints_int, int* use_arithmetic_constraints_int,
                                   int* use_adaptive_constraints_int, int* use_user_constraints_int,
                                   int* weights_type) {
  guarded("bddcml_setup_preconditioner_c", [&] {
    Solver* S = need_solver("bddcml_setup_preconditioner_c");
    if (!S) return;
    (void)parallel_division_int;
    S->prm.matrixtype = *matrixtype;
    if (use_defaults_int && *use_defaults_int) {  // module_bddcml.f90:411-416
      S->prm.use_corner = true; S->prm.use_arith = true; S->prm.use_adaptive = false; S->prm.use_user = false;
      S->prm.weights_type = 0;
    } else {
      S->prm.use_corner = *use_corner_constraints_int != 0;
      S->prm.use_arith = *use_arithmetic_constraints_int != 0;
      S->prm.use_adaptive = *use_adaptive_constraints_int != 0;
      S->prm.use_user = *use_user_constraints_int != 0;
      S->prm.weights_type = *weights_type;
    }
    if (S->prm.use_adaptive && !S->prm.use_arith)  // an add-on to the arithmetic ones (module_levels.f90:2699-2700)
      throw Error{ERR_UNSUPPORTED, "adaptive constraints need the arithmetic face constraints"};
    if (S->prm.use_adaptive && S->prm.matrixtype != 1)
      throw Error{ERR_UNSUPPORTED, "adaptive constraints are implemented for SPD matrices (matrixtype 1)"};
    if (S->prm.use_user) throw Error{ERR_UNSUPPORTED, "user constraints are not implemented"};
    for (auto& sd : S->subs)
      if (sd.loaded && (sd.matrixtype == 0) != (S->prm.matrixtype == 0))
        throw Error{ERR_ARGUMENT, "matrixtype differs from the one of the uploaded subdomain matrices"};
    if (S->prm.matrixtype == 0 && S->prm.nlevels == 3)
      throw Error{ERR_UNSUPPORTED, "three levels are implemented for symmetric matrices"};
    double t0 = wall_time();
    S->stats = Stats{};
    S->stats.t_upload = S->t_upload;
    if (S->global.present && !S->subs.empty() && !S->subs[0].loaded) {
      host_localize_global(*S, *matrixtype);  // global loading: divide and localise now
      for (auto& sd : S->subs) sd.matrixtype = *matrixtype;
    }
    host_setup(*S);
    S->stats.t_host_setup = wall_time() - t0;
    if (!S->dev) {
      Error err{0, ""};
      S->dev = device_create(err);
      if (!S->dev) throw err;
    }
    device_set_profiling(S->dev, S->profiling);
    Error err{0, ""};
    if (!device_setup(*S, err)) throw err;
    S->setup_done = true;
  });
}

void bddcml_solve_c(int* comm_all, int* method, double* tol, int* maxit, int* ndecrmax, int* recycling_int,
                    int* max_number_of_stored_vectors, int* num_iter, int* converged_reason,
                    double* condition_number) {
  guarded("bddcml_solve_c", [&] {
    (void)comm_all;
    Solver* S = need_solver("bddcml_solve_c");
    if (!S) return;
    if (!S->setup_done) throw Error{ERR_ARGUMENT, "preconditioner is not set up"};
    // method -1 takes the reference defaults (module_bddcml.f90:515-520, 544-567):
    // BiCGSTAB, tol 1e-6, maxit 1000, ndecrmax 30
    int m = 1, mi = 1000, nd = 30;
    double t = 1e-6;
    if (*method != -1) { m = *method; t = *tol; mi = *maxit; nd = *ndecrmax; }
    if (m == 5) throw Error{ERR_UNSUPPORTED, "method 5 (direct solve by backsubstitution) is not implemented"};
    if (m < 0 || m > 2) throw Error{ERR_ARGUMENT, "unknown iterative method " + std::to_string(m)};
    if (mi < 1) throw Error{ERR_ARGUMENT, "maxit must be positive"};
    int it = 0, reason = 0;
    double cond = 1.0;
    Error err{0, ""};
    // Krylov recycling is part of PCG only (module_bddcml.f90:544-567); the reference's
    // defaults switch it off (module_bddcml.f90:519-520)
    int rec = 0, maxvec = 0;
    if (*method != -1 && m == 0) {
      rec = *recycling_int;
      maxvec = *max_number_of_stored_vectors;
      if (rec && maxvec < 0) throw Error{ERR_ARGUMENT, "max_number_of_stored_vectors must not be negative"};
    }
    if (!device_solve(*S, m, t, mi, nd, rec, maxvec, it, reason, cond, err)) throw err;
    S->solved = true;
    S->reactions_ready = false;
    *num_iter = it;
    *converged_reason = reason;
    *condition_number = cond;
  });
}

// ---------------------------------------------------------- batched loads
// Extension: nrhs loads of the same set-up problem solved by one batched PCG.
void bddcml_upload_subdomain_rhs_batch_c(int* isub, int* nrhs, double* rhss, int* lrhss, int* is_rhs_complete) {
  guarded("bddcml_upload_subdomain_rhs_batch_c", [&] {
    Solver* S = need_solver("bddcml_upload_subdomain_rhs_batch_c");
    if (!S) return;
    int t = sub_index(*S, *isub);
    Subdomain& s = S->subs[t];
    if (!s.loaded) throw Error{ERR_ARGUMENT, "the subdomain data must be uploaded first"};
    if (*nrhs < 1 || *nrhs > 64) throw Error{ERR_ARGUMENT, "nrhs must be between 1 and 64"};
    if ((long long)*lrhss != (long long)s.ndof * *nrhs) throw Error{ERR_ARGUMENT, "lrhss must be ndof * nrhs"};
    s.rhs_batch.assign(rhss, rhss + *lrhss);
    s.nrhs_batch = *nrhs;
    s.rhs_batch_complete = is_rhs_complete && *is_rhs_complete != 0;
  });
}

void bddcml_solve_batch_c(int* comm_all, int* method, double* tol, int* maxit, int* ndecrmax, int* nrhs,
                          int* num_iter, int* converged_reason, double* condition_number) {
  guarded("bddcml_solve_batch_c", [&] {
    (void)comm_all;
    Solver* S = need_solver("bddcml_solve_batch_c");
    if (!S) return;
    if (!S->setup_done) throw Error{ERR_ARGUMENT, "preconditioner is not set up"};
    if (*method != 0) throw Error{ERR_UNSUPPORTED, "batched right-hand sides are solved by PCG (method 0) only"};
    if (S->prm.matrixtype == 0) throw Error{ERR_UNSUPPORTED, "batched solves need a symmetric matrix (PCG)"};
    if (*maxit < 1) throw Error{ERR_ARGUMENT, "maxit must be positive"};
    if (*nrhs < 1 || *nrhs > 64) throw Error{ERR_ARGUMENT, "nrhs must be between 1 and 64"};
    for (auto& s : S->subs)
      if (s.nrhs_batch != *nrhs)
        throw Error{ERR_ARGUMENT, "every subdomain needs nrhs right-hand sides from bddcml_upload_subdomain_rhs_batch"};
    vector<int> it, reason;
    vector<double> cond;
    Error err{0, ""};
    S->batch_solved = 0;
    if (!device_solve_batch(*S, *nrhs, *tol, *maxit, *ndecrmax, it, reason, cond, err)) throw err;
    S->batch_solved = *nrhs;
    for (int k = 0; k < *nrhs; ++k) {
      num_iter[k] = it[k];
      converged_reason[k] = reason[k];
      condition_number[k] = cond[k];
    }
  });
}

void bddcml_set_batch_operator_c(int* mode) {
  guarded("bddcml_set_batch_operator_c", [&] {
    Solver* S = need_solver("bddcml_set_batch_operator_c");
    if (!S) return;
    if (*mode < -1 || *mode > 2) throw Error{ERR_ARGUMENT, "batch operator mode must be -1, 0, 1 or 2"};
    S->prm.batch_operator = *mode;
  });
}

void bddcml_download_local_solution_batch_c(int* isub, int* nrhs, double* sols, int* lsols) {
  guarded("bddcml_download_local_solution_batch_c", [&] {
    Solver* S = need_solver("bddcml_download_local_solution_batch_c");
    if (!S) return;
    if (S->batch_solved == 0 || *nrhs != S->batch_solved)
      throw Error{ERR_ARGUMENT, "no batched solve with nrhs right-hand sides"};
    int t = sub_index(*S, *isub);
    Subdomain& s = S->subs[t];
    if ((long long)*lsols != (long long)s.ndof * *nrhs) throw Error{ERR_ARGUMENT, "lsols must be ndof * nrhs"};
    std::copy(s.sol_batch.begin(), s.sol_batch.end(), sols);
  });
}

void bddcml_download_local_solution_c(int* isub, double* sols, int* lsols) {
  guarded("bddcml_download_local_solution_c", [&] {
    Solver* S = need_solver("bddcml_download_local_solution_c");
    if (!S) return;
    int t = sub_index(*S, *isub);
    Subdomain& s = S->subs[t];
    if (*lsols != s.ndof) throw Error{ERR_ARGUMENT, "lsols does not match the subdomain dof count"};
    std::copy(s.sol.begin(), s.sol.end(), sols);
  });
}

// the global vector with every subdomain's values written at its global dofs,
// subdomains in order (levels_get_global_solution, module_levels.f90:4617-4744)
static void gather_global(const Solver& S, const vector<double> Subdomain::*field, double* out, int lout) {
  if (lout != S.ndof_global) throw Error{ERR_ARGUMENT, "array length does not match the global dof count"};
  std::fill(out, out + lout, 0.0);
  for (auto& s : S.subs) {
    const vector<double>& v = s.*field;
    for (int i = 0; i < s.ndof; ++i) out[s.isvgvn[i]] = v[i];
  }
}

static void need_reactions(Solver& S) {
  if (!S.solved) throw Error{ERR_ARGUMENT, "reactions are available after bddcml_solve"};
  if (S.prm.matrixtype == 0) throw Error{ERR_UNSUPPORTED, "reactions are implemented for symmetric matrices"};
  if (!S.reactions_ready) {
    host_reactions(S);
    S.reactions_ready = true;
  }
}

void bddcml_download_global_solution_c(double* sol, int* lsol) {
  guarded("bddcml_download_global_solution_c", [&] {
    Solver* S = need_solver("bddcml_download_global_solution_c");
    if (!S) return;
    gather_global(*S, &Subdomain::sol, sol, *lsol);
  });
}

void bddcml_download_local_reactions_c(int* isub, double* reas, int* lreas) {
  guarded("bddcml_download_local_reactions_c", [&] {
    Solver* S = need_solver("bddcml_download_local_reactions_c");
    if (!S) return;
    int t = sub_index(*S, *isub);
    need_reactions(*S);
    Subdomain& s = S->subs[t];
    if (*lreas != s.ndof) throw Error{ERR_ARGUMENT, "lreas does not match the subdomain dof count"};
    std::copy(s.rea.begin(), s.rea.end(), reas);
  });
}

void bddcml_download_global_reactions_c(double* rea, int* lrea) {
  guarded("bddcml_download_global_reactions_c", [&] {
    Solver* S = need_solver("bddcml_download_global_reactions_c");
    if (!S) return;
    need_reactions(*S);
    gather_global(*S, &Subdomain::rea, rea, *lrea);
  });
}

// new fixed values, loads and initial guess of globally loaded data
// (levels_change_global_data): restricted to the subdomains of the division
// made at setup, as bddcml_change_subdomain_data_c does per subdomain
void bddcml_change_global_data_c(int* ifix, int* lifix, double* fixv, int* lfixv, double* rhs, int* lrhs,
                                 double* sol, int* lsol) {
  guarded("bddcml_change_global_data_c", [&] {
    Solver* S = need_solver("bddcml_change_global_data_c");
    if (!S) return;
    GlobalData& G = S->global;
    if (!G.present)
      throw Error{ERR_UNSUPPORTED, "global data must be loaded by bddcml_upload_global_data_file_c"};
    if (!S->setup_done) throw Error{ERR_ARGUMENT, "data can be changed only after bddcml_setup_preconditioner"};
    if (*lifix != G.ndof || *lfixv != G.ndof || *lrhs != G.ndof || *lsol != G.ndof)
      throw Error{ERR_ARGUMENT, "array length does not match the global dof count"};
    for (int q = 0; q < G.ndof; ++q)
      if ((ifix[q] != 0) != (G.ifix[q] != 0))
        throw Error{ERR_UNSUPPORTED, "the set of fixed dofs changed; that needs a new setup"};
    G.fixv.assign(fixv, fixv + G.ndof);
    G.rhs.assign(rhs, rhs + G.ndof);
    G.sol.assign(sol, sol + G.ndof);
    for (auto& s : S->subs) {
      for (int q = 0; q < s.ndof; ++q) {
        const int g = s.isvgvn[q];
        s.fixv[q] = G.fixv[g];
        s.rhs[q] = G.rhs[g];
        s.sol[q] = G.sol[g];
      }
      s.rhs_complete = true;
    }
    S->new_data_pending = true;
  });
}

void bddcml_change_subdomain_data_c(int* isub, int* ifix, int* lifix, double* fixv, int* lfixv, double* rhs,
                                    int* lrhs, int* is_rhs_complete, double* sol, int* lsol) {
  guarded("bddcml_change_subdomain_data_c", [&] {
    Solver* S = need_solver("bddcml_change_subdomain_data_c");
    if (!S) return;
    if (!S->setup_done) throw Error{ERR_ARGUMENT, "data can be changed only after bddcml_setup_preconditioner"};
    int t = sub_index(*S, *isub);
    Subdomain& s = S->subs[t];
    if (*lifix != s.ndof || *lfixv != s.ndof || *lrhs != s.ndof || *lsol != s.ndof)
      throw Error{ERR_ARGUMENT, "array length does not match ndofs of the subdomain"};
    // the eliminated matrix and the coarse space depend on which dofs are
    // fixed; only the values may change (module_levels.f90:785-853)
    for (int i = 0; i < s.ndof; ++i)
      if ((ifix[i] != 0) != (s.ifix[i] != 0))
        throw Error{ERR_UNSUPPORTED, "the set of fixed dofs changed; that needs a new setup"};
    s.fixv.assign(fixv, fixv + s.ndof);
    s.rhs.assign(rhs, rhs + s.ndof);
    s.rhs_complete = is_rhs_complete && *is_rhs_complete != 0;
    s.sol.assign(sol, sol + s.ndof);
    S->new_data_pending = true;
  });
}

void bddcml_setup_new_data_c(void) {
  guarded("bddcml_setup_new_data_c", [&] {
    Solver* S = need_solver("bddcml_setup_new_data_c");
    if (!S) return;
    if (!S->setup_done) throw Error{ERR_ARGUMENT, "bddcml_setup_preconditioner must come first"};
    host_new_data(*S);
    Error err{BDDCML_OK, ""};
    if (!device_new_data(*S, err)) throw err;
    S->new_data_pending = false;
  });
}

void bddcml_dotprod_subdomain_c(int* isub, double* vec1, int* lvec1, double* vec2, int* lvec2, double* dotprod) {
  guarded("bddcml_dotprod_subdomain_c", [&] {
    Solver* S = need_solver("bddcml_dotprod_subdomain_c");
    if (!S) return;
    int t = sub_index(*S, *isub);
    Subdomain& s = S->subs[t];
    if (s.wi.empty() && s.ndofi > 0) throw Error{ERR_ARGUMENT, "weights are not ready"};
    if (*lvec1 != *lvec2 || *lvec1 != s.ndof) throw Error{ERR_ARGUMENT, "dimension mismatch"};
    double d = 0.0;  // module_dd.f90:12736-12788
    for (int i = 0; i < s.ndofi; ++i) d += vec1[s.iivsvn[i]] * s.wi[i] * vec2[s.iivsvn[i]];
    for (int i = 0; i < s.ndofo; ++i) d += vec1[s.iovsvn[i]] * vec2[s.iovsvn[i]];
    *dotprod = d;
  });
}

void bddcml_finalize_c(void) {
  guarded("bddcml_finalize_c", [&] {
    g_solver.reset();  // the solver destroys its device state
  });
}

void bddcml_dotprod_subdomain_dev_c(int* isub, const double* vec1, const double* vec2, int* lvec, double* dotprod) {
  guarded("bddcml_dotprod_subdomain_dev_c", [&] {
    Solver* S = need_solver("bddcml_dotprod_subdomain_dev_c");
    if (!S) return;
    int t = sub_index(*S, *isub);
    Subdomain& s = S->subs[t];
    if (s.wi.empty() && s.ndofi > 0) throw Error{ERR_ARGUMENT, "weights are not ready"};
    if (*lvec != s.ndof) throw Error{ERR_ARGUMENT, "dimension mismatch"};
    Error err{BDDCML_OK, ""};
    if (!device_dotprod_noalloc(s.iivsvn.data(), s.wi.data(), s.ndofi, vec1, vec2, s.ndof, dotprod, err)) throw err;
  });
}

void bddcml_element_gradient_dev_c(int* nelem, int* nne, const int* inet, const double* ke0, int* ke0_per_element,
                                   const double* u, const double* lam, double* grad) {
  guarded("bddcml_element_gradient_dev_c", [&] {
    if (!nelem || !nne || !ke0_per_element) throw Error{ERR_ARGUMENT, "null size argument"};
    Error err{BDDCML_OK, ""};
    if (!device_element_gradient(*nelem, *nne, inet, ke0, *ke0_per_element != 0, u, lam, grad, err)) throw err;
  });
}

void bddcml_release_device_memory_c(void) {
  guarded("bddcml_release_device_memory_c", [&] {
    Error err{BDDCML_OK, ""};
    if (!device_release_memory(err)) throw err;
  });
}

void bddcml_set_wait_limit_c(long long* spins) {
  guarded("bddcml_set_wait_limit_c", [&] {
    Error err{BDDCML_OK, ""};
    if (!device_set_wait_limit(*spins, err)) throw err;
  });
}

int bddcml_get_last_error_c(char* msg, int* lmsg) {
  if (msg && lmsg && *lmsg > 0) {
    int n = std::min<int>((int)g_msg.size(), *lmsg - 1);
    std::memcpy(msg, g_msg.data(), n);
    msg[n] = '\0';
  }
  return g_status;
}

void bddcml_set_precision_c(int* mode) {
  guarded("bddcml_set_precision_c", [&] {
    Solver* S = need_solver("bddcml_set_precision_c");
    if (!S) return;
    if (*mode != 0 && *mode != 1) throw Error{ERR_ARGUMENT, "precision mode must be 0 (FP64) or 1 (mixed)"};
    S->prm.precision = *mode;
  });
}

void bddcml_get_stats_c(double* stats, int* lstats) {
  guarded("bddcml_get_stats_c", [&] {
    Solver* S = need_solver("bddcml_get_stats_c");
    if (!S) return;
    const Stats& q = S->stats;
    double v[] = {q.t_host_setup, q.t_device_setup, q.t_solve, q.t_iterations, q.t_postprocess,
                  (double)q.num_iter, q.bytes_per_iteration, (double)q.ncorner, (double)q.nedge, (double)q.nface,
                  (double)q.ndofc, (double)q.sum_ndofi, (double)q.sum_ndofo, (double)q.ninterface,
                  (double)S->prm.precision, q.h2d_bytes, q.d2h_bytes, q.t_upload, q.t_host_assemble,
                  q.t_host_iface, q.t_host_globs, q.t_host_blocks, q.refine1, q.refine2,
                  q.flop_sweep_oo, q.flop_sweep_s, q.bytes_residual, q.bytes_schur_apply, q.bytes_pc_local,
                  q.launches_setup, q.launches_solve, q.t_dev_alloc, q.t_dev_h2d, (double)q.npair,
                  (double)q.nadaptive, q.adapt_est, q.t_adaptive, q.lobpcg_resid, (double)q.lobpcg_iter,
                  q.batch_bytes_schur, q.batch_flop_schur_mma, q.batch_flop_schur, q.batch_flop_pc, q.batch_nk,
                  q.bytes_assemble_dot, q.bytes_assemble_z, q.bytes_coarse_apply, q.refine_steps, q.band_w};
    int n = std::min<int>(*lstats, (int)(sizeof(v) / sizeof(v[0])));
    for (int i = 0; i < n; ++i) stats[i] = v[i];
    *lstats = n;
  });
}

void bddcml_set_adaptive_threshold_c(double* tau) {
  guarded("bddcml_set_adaptive_threshold_c", [&] {
    Solver* S = need_solver("bddcml_set_adaptive_threshold_c");
    if (!S) return;
    if (!(*tau > 0.0)) throw Error{ERR_ARGUMENT, "the adaptive threshold must be positive"};
    S->prm.adaptive_tau = *tau;
  });
}

void bddcml_get_adaptive_info_c(int* pairs, double* eigs, int* lpair) {
  guarded("bddcml_get_adaptive_info_c", [&] {
    Solver* S = need_solver("bddcml_get_adaptive_info_c");
    if (!S) return;
    const AdaptivePairs& P = S->adaptive_pairs;
    const int n = std::min(*lpair, P.npair);
    for (int p = 0; p < n; ++p) {
      pairs[3 * p + 0] = P.si[p] + S->prm.numbase;
      pairs[3 * p + 1] = P.sj[p] + S->prm.numbase;
      pairs[3 * p + 2] = P.k[p];
      for (int c = 0; c < AdaptivePairs::KMAX; ++c)
        eigs[(size_t)p * AdaptivePairs::KMAX + c] =
            c < P.k[p] ? S->adaptive_eigs[(size_t)p * AdaptivePairs::KMAX + c] : 0.0;
    }
    *lpair = P.npair;
  });
}

void bddcml_get_residual_history_c(double* hist, int* lhist) {
  guarded("bddcml_get_residual_history_c", [&] {
    Solver* S = need_solver("bddcml_get_residual_history_c");
    if (!S) return;
    int n = std::min<int>(*lhist, (int)S->relres_history.size());
    for (int i = 0; i < n; ++i) hist[i] = S->relres_history[i];
    *lhist = (int)S->relres_history.size();
  });
}

void bddcml_get_interface_weights_c(int* isub, double* wi, int* lwi) {
  guarded("bddcml_get_interface_weights_c", [&] {
    Solver* S = need_solver("bddcml_get_interface_weights_c");
    if (!S) return;
    int t = sub_index(*S, *isub);
    Subdomain& s = S->subs[t];
    if (*lwi != (int)s.wi.size()) throw Error{ERR_ARGUMENT, "lwi does not match ndofi"};
    std::copy(s.wi.begin(), s.wi.end(), wi);
  });
}

void bddcml_set_profiling_c(int* on) {
  guarded("bddcml_set_profiling_c", [&] {
    Solver* S = need_solver("bddcml_set_profiling_c");
    if (!S) return;
    S->profiling = *on != 0;
    if (S->dev) device_set_profiling(S->dev, S->profiling);
  });
}

void bddcml_get_profile_c(double* ms, int* counts, int* lphase) {
  guarded("bddcml_get_profile_c", [&] {
    Solver* S = need_solver("bddcml_get_profile_c");
    if (!S) return;
    double m[NPHASE] = {0};
    int c[NPHASE] = {0};
    if (S->dev) device_get_profile(S->dev, m, c);
    int n = std::min<int>(*lphase, NPHASE);
    for (int i = 0; i < n; ++i) { ms[i] = m[i]; counts[i] = c[i]; }
    *lphase = NPHASE;
  });
}

void bddcml_get_setup_digest_c(unsigned long long* digest) {
  guarded("bddcml_get_setup_digest_c", [&] {
    Solver* S = need_solver("bddcml_get_setup_digest_c");
    if (!S) return;
    if (!digest) throw Error{ERR_ARGUMENT, "null argument"};
    // FNV-1a over the bytes of every host-side setup result, in subdomain order
    unsigned long long h = 1469598103934665603ull;
    auto bytes = [&h](const void* p, size_t n) {
      const unsigned char* c = static_cast<const unsigned char*>(p);
      for (size_t i = 0; i < n; ++i) { h ^= c[i]; h *= 1099511628211ull; }
    };
    auto arr = [&](const auto& v) {
      const unsigned long long n = v.size();
      bytes(&n, sizeof n);
      if (n) bytes(v.data(), n * sizeof(v[0]));
    };
    auto val = [&](const auto& x) { bytes(&x, sizeof x); };
    for (const auto& s : S->subs) {
      arr(s.ia); arr(s.ja); arr(s.a); arr(s.comp);
      arr(s.iin); arr(s.kdofi); arr(s.iivsvn); arr(s.iovsvn); arr(s.adj);
      for (const auto& cn : s.cnodes) {
        val(cn.itype); val(cn.global_number); arr(cn.inodi); arr(cn.idofi); val(cn.ncdof); val(cn.used);
        arr(cn.matrix);
      }
      arr(s.c_ptr); arr(s.c_col); arr(s.c_val); arr(s.indrowc);
      arr(s.bc); arr(s.bcx_tgt); arr(s.bcx_src); arr(s.bcx_val); arr(s.fxr_i); arr(s.fxr_j); arr(s.fxr_v);
      arr(s.wi); arr(s.uniq); arr(s.operm); val(s.band);
    }
    int v[] = {S->ncorner, S->nedge, S->nface, S->ndofc, S->ninterface};
    bytes(v, sizeof v);
    *digest = h;
  });
}

void bddcml_get_coarse_info_c(int* out, int* lout) {
  guarded("bddcml_get_coarse_info_c", [&] {
    Solver* S = need_solver("bddcml_get_coarse_info_c");
    if (!S) return;
    long si = 0, so = 0;
    for (auto& s : S->subs) { si += s.ndofi; so += s.ndofo; }
    int v[] = {S->ncorner, S->nedge, S->nface, S->ndofc, (int)si, (int)so};
    int n = std::min<int>(*lout, 6);
    for (int i = 0; i < n; ++i) out[i] = v[i];
    *lout = n;
  });
}

}  // extern "C"
