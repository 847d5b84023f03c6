// Internal data model of the GB300 BDDC solver (host side).
//
// One process, one GPU, every subdomain resident on the device.  The host
// keeps the uploaded subdomain data (module_dd.f90:65-372 subdomain_type is the
// reference's equivalent) and runs the integer/geometric part of the setup:
// interface detection, globs and corners, coarse numbering, Dirichlet
// elimination and weights.  Everything numeric after that runs on the GPU.
#pragma once

#include <array>
#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace bddc {

using std::vector;

// allocator whose resize leaves new elements uninitialised: the uploaded
// triplets are written once by a parallel copy, and a zero fill before it
// would be a second serial pass over the largest input
template <class T>
struct NoInitAllocator : std::allocator<T> {
  template <class U>
  struct rebind { using other = NoInitAllocator<U>; };
  NoInitAllocator() = default;
  template <class U>
  NoInitAllocator(const NoInitAllocator<U>&) noexcept {}
  template <class U>
  void construct(U* p) noexcept { ::new ((void*)p) U; }
  template <class U, class... A>
  void construct(U* p, A&&... a) { ::new ((void*)p) U(std::forward<A>(a)...); }
};
template <class T>
using rawvec = std::vector<T, NoInitAllocator<T>>;

// status codes (mirror include/bddcml_gb300.h)
enum Status { OK = 0, ERR_ARGUMENT = 1, ERR_CUDA = 2, ERR_NUMERIC = 3, ERR_UNSUPPORTED = 4, ERR_MEMORY = 5 };

// timed phases (CUDA events on the solver stream); order is part of the
// bddcml_get_profile_c extension
enum Phase {
  PH_NUMERIC_TOTAL = 0, PH_SOLVE_TOTAL, PH_FACTOR_OO, PH_SOLVE_OO, PH_RESIDUAL, PH_SCHUR, PH_SRHO_FACTOR,
  PH_SRHO_SOLVE, PH_PC_BLOCKS, PH_COARSE, PH_PCG, PH_SCHUR_APPLY, PH_PC_LOCAL, PH_POST, PH_ASSEMBLE_DOT,
  PH_ASSEMBLE_Z, PH_COARSE_APPLY, NPHASE
};

struct Error {
  int code;
  std::string msg;
};

// one coarse node of a subdomain: a corner, an edge or a face
// (module_dd.f90:43-62 cnode_type)
struct CoarseNode {
  int itype = 0;          // 3 corner, 2 edge, 1 face
  int global_number = 0;  // 1-based over corners, then edges, then faces
  vector<int> inodi;      // interface nodes of the glob
  vector<int> idofi;      // interface dofs of the glob
  int ncdof = 0;          // number of constraint rows it contributes
  bool used = false;
  // explicit rows (ncdof x idofi.size(), row-major) once the face constraints
  // have been made adaptive; empty = the corner / arithmetic-average rows
  vector<double> matrix;
};

struct Subdomain {
  // ---------------- uploaded (0-based local numbering)
  int nelem = 0, nnod = 0, ndof = 0, ndim = 0;
  vector<int> inet, nnet, nndf, isngn, isvgvn, isegn, ifix;
  vector<double> xyz;  // column-major (nnod x ndim)
  vector<double> fixv, rhs, sol;
  bool rhs_complete = true;
  // batched right-hand sides (ndof x nrhs_batch, column-major) and their solutions
  vector<double> rhs_batch, sol_batch;
  int nrhs_batch = 0;
  bool rhs_batch_complete = true;
  int matrixtype = 1;
  rawvec<int> ia, ja;  // upper triangle (merged at setup)
  rawvec<double> a;
  bool loaded = false;
  bool assembled = false;
  bool find_components = true;
  bool dual_graph = true;
  int neighbouring = 1;

  // ---------------- derived on the host
  bool bc_present = false;
  vector<int> comp;          // nodal components, 1-based
  vector<int> kdof;          // first dof of each node
  vector<int> iin;           // interface nodes (local order)
  vector<int> kdofi;         // first interface dof of each interface node (nnodi+1)
  vector<int> iivsvn;        // interface dofs (local dof index)
  vector<int> iovsvn;        // interior dofs (local dof index)
  int nnodi = 0, ndofi = 0, ndofo = 0;
  vector<int> adj;           // neighbour subdomains, ascending (0-based)
  vector<CoarseNode> cnodes;
  // constraints in CSR over interface dofs; indrowc = global coarse dof (0-based)
  vector<int> c_ptr, c_col;
  vector<double> c_val;
  vector<int> indrowc;
  int nconstr = 0;
  vector<double> bc;         // eliminated Dirichlet contributions, interface assembled
  // the elimination as a replayable list: bc[bcx_tgt] += bcx_val * fixv[bcx_src],
  // in the order the first elimination applied them (the reference keeps the
  // fixed rows of the matrix for the same purpose, module_dd.f90:1081-1180)
  vector<int> bcx_tgt, bcx_src;
  vector<double> bcx_val;
  // entries of the uploaded matrix in fixed rows or columns, kept before the
  // elimination for the reactions (the fixed-rows matrix of module_dd.f90:1160-1211)
  vector<int> fxr_i, fxr_j;
  vector<double> fxr_v;
  vector<double> rea;        // reactions after the last solve
  vector<double> wi;         // interface weights
  vector<double> rhoi;       // coefficients the weights are built from (module_dd.f90:11660-11722)
  vector<int> uniq;          // interface dof -> unique interface index
  // interior ordering used for the band factor: perm[new] = index into iovsvn
  vector<int> operm;
  int band = 0;              // half bandwidth of the reordered interior block
  double rho = 1.0;          // scale of the constraint penalty in the preconditioner
};

struct Params {
  int nlevels = 2;
  int nsub = 0;
  int nsub2 = 1;              // subdomains of level 2 (three levels)
  int numbase = 0;
  int verbose = 0;
  int precision = 1;          // 0 plain FP64, 1 mixed
  // preconditioner options
  bool use_corner = true, use_arith = true, use_adaptive = false, use_user = false;
  int weights_type = 0;
  int matrixtype = 1;
  double adaptive_tau = 1.5;  // eigenvalue threshold of adaptive constraints (module_adaptivity.f90:30)
  int batch_operator = -1;    // batched products in mixed mode (bddcml_set_batch_operator_c): -1 automatic, 0, 1, 2
};

struct Stats {
  double t_host_setup = 0, t_device_setup = 0, t_solve = 0, t_factor = 0, t_schur = 0, t_precond = 0,
         t_coarse = 0, t_iterations = 0, t_postprocess = 0;
  double bytes_per_iteration = 0;
  int ncorner = 0, nedge = 0, nface = 0, ndofc = 0;
  long long sum_ndofi = 0, sum_ndofo = 0, ninterface = 0;
  int num_iter = 0;
  double setup_flops = 0;
  double h2d_bytes = 0, d2h_bytes = 0;
  double t_upload = 0, t_host_assemble = 0, t_host_iface = 0, t_host_globs = 0, t_host_blocks = 0;
  double refine1 = 0, refine2 = 0;  // max |correction| / max |X| of the first and the last refinement step
  double refine_steps = 0;          // refinement steps of the interior solves
  double band_w = 0;                // largest block bandwidth of the interior systems
  // batched solve, per Schur / preconditioner apply: operator bytes streamed, tensor-core
  // flops executed (sliced operator), FP64-equivalent flops of S X, working-precision
  // flops of the local preconditioner products, and the batch width
  double batch_bytes_schur = 0, batch_flop_schur_mma = 0, batch_flop_schur = 0, batch_flop_pc = 0, batch_nk = 0;
  // algorithmic work per launch of the main phases (for roofline reporting)
  double flop_sweep_oo = 0;     // one forward + backward interior sweep, all subdomains (FP32 flop)
  double flop_sweep_s = 0;      // one forward + backward preconditioner-block sweep
  double bytes_residual = 0;    // one refinement residual (X read once, R written)
  double bytes_schur_apply = 0; // one Schur operator apply
  double bytes_pc_local = 0;    // one local preconditioner apply
  // interface kernels of a PCG iteration: assembly of S p with the dot product
  // (k_assemble_dot), assembly of z with the coarse correction (k_assemble_z),
  // and the two-level coarse solve (gather, inverse, two refinements)
  double bytes_assemble_dot = 0, bytes_assemble_z = 0, bytes_coarse_apply = 0;
  double launches_setup = 0, launches_solve = 0;  // kernel launches of the last set-up / solve
  double t_dev_alloc = 0, t_dev_h2d = 0;  // device set-up: allocations, staging + host->device copies
  // adaptive face constraints
  int npair = 0, nadaptive = 0, lobpcg_iter = 0;
  double adapt_est = -1, t_adaptive = 0, lobpcg_resid = 0;
};

// Face pairs of the adaptive constraint search (module_adaptivity.f90): the
// space of both interfaces of a face's two subdomains, n = ni + nj rows
// (first subdomain's interface dofs, then the second's).
struct AdaptivePairs {
  static constexpr int KMAX = 10;  // neigvecx, module_adaptivity.f90:44
  int npair = 0;
  vector<int> si, sj, fi, fj;      // subdomains and the face coarse node in each
  vector<int> ni, n, m, k;         // first interface size, pair size, Q columns, eigenvectors
  vector<int> md;                  // columns of Q from D (the rest span null(S) within null(D))
  vector<long long> vo, qo;        // offsets of the pair's vector block (n x KMAX) and of Q (n x m)
  vector<int> cptr;                // common dofs of pair p: [cptr[p], cptr[p + 1])
  vector<int> ca, cb;              // their rows in the pair space (cb counts from 0 of the pair)
  vector<double> wa, wb;           // weights rho_a / (rho_a + rho_b), rho_b / (rho_a + rho_b)
  vector<double> q;                // orthonormal basis of range(D^T), column-major per pair
  long long nvec = 0, nq = 0;      // total rows x KMAX, total Q entries
};

// Per-subdomain matrix blocks in device-ready form (interior rows in the
// band-reducing order): A_oo, A_oi, A_io, A_ii as CSR, the reduced-rhs inputs
// and the band width of A_oo in 64-row blocks.
struct SubBlocks {
  vector<int> oo_ptr, oi_ptr, io_ptr, ii_ptr;
  rawvec<int> oo_col, oi_col, io_col, ii_col;  // written once by the row split: no zero fill
  rawvec<double> oo_val, oi_val, io_val, ii_val;
  vector<double> fo, fi;  // interior rhs (new order), interface rhs (weighted)
  int w = 0;
  double rho = 1.0;
  int maxrow_oo = 0, maxrow_oi = 0, maxrow_io = 0, maxrow_ii = 0;
};

class Device;  // GPU side (bddc_device.cu)

// global mesh and data uploaded as a whole (levels_upload_global_data,
// module_levels.f90:422-612), localised to the subdomains at setup
struct GlobalData {
  bool present = false;
  int nelem = 0, nnod = 0, ndof = 0, ndim = 0, meshdim = 0, neighbouring = 1;
  vector<int> inet, nnet, nndf, ifix;  // 0-based node numbers in inet
  vector<double> xyz, fixv, rhs, sol;   // xyz column-major (nnod x ndim)
  std::string elm_file;                 // Fortran unformatted element matrices, one record per element
};

struct Solver {
  Params prm;
  vector<Subdomain> subs;
  GlobalData global;
  int nelem = 0, nnod = 0, ndof_global = 0;
  // coarse space
  int ncorner = 0, nedge = 0, nface = 0, ndofc = 0;
  // unique interface numbering
  int ninterface = 0;                 // number of unique interface dofs
  vector<int> iface_fixed;            // per unique dof: 1 if Dirichlet-fixed
  vector<double> iface_wsum;          // per unique dof: sum of subdomain weights
  bool setup_done = false;
  bool new_data_pending = false;  // changed subdomain data not yet through setup_new_data
  int batch_solved = 0;           // right-hand sides of the last batched solve (0: none)
  bool solved = false;            // a solve has produced the subdomain solutions
  bool reactions_ready = false;   // reactions computed for the last solve
  Device* dev = nullptr;
  Stats stats;
  vector<double> relres_history;
  bool profiling = false;
  double t_upload = 0;              // accumulated time inside the upload calls
  vector<SubBlocks> blocks;         // device-ready blocks, freed after upload
  // last adaptive constraint search: the pairs and their eigenvalues (KMAX per pair)
  AdaptivePairs adaptive_pairs;
  vector<double> adaptive_eigs;
  // three levels: the level-2 problem (its own host data and device state)
  std::unique_ptr<Solver> lev2;
  ~Solver();
};

// adaptive face constraints, host part (bddc_adaptive.cpp)
// nulls[s]: orthonormal basis of null(S_s) on the interface (ndofi x d_s, column-major; empty if none)
void host_adaptive_pairs(const Solver& S, AdaptivePairs& P, const vector<vector<double>>& nulls);
// null space coefficients of a local coarse matrix Phi^T S Phi (nc x nc in an ld x ld array):
// the eigenvectors with |eigenvalue| <= nc * max |eigenvalue| * 4 * 2^-44, nc x d column-major
vector<double> host_coarse_null_coefficients(int nc, int ld, const double* ac, int& d);
// eig: npair x KMAX eigenvalues (descending); cons: for every pair the columns A x of the
// eigenvectors with eigenvalue >= tau, n rows each, packed pair after pair
void host_load_adaptive(Solver& S, const AdaptivePairs& P, const vector<double>& eig, const vector<double>& cons);
// global coarse numbering and the constraint rows of every subdomain from its coarse nodes
void host_constraint_rows(Solver& S);

// three-level BDDC (bddc_levels.cpp): division of the level-1 subdomains and the level-2
// problem built from the level-1 coarse space; acs[s] = local coarse matrix of s (nc x nc)
vector<int> host_level_division(const vector<std::array<double, 3>>& centroids, int ndim, int nparts);
// global data to subdomain data: element division, local numbering, element
// matrices from the ELM file (bddc_global.cpp)
void host_localize_global(Solver& S, int matrixtype);
std::unique_ptr<Solver> host_build_level2(const Solver& S1, const vector<vector<double>>& acs, int nsub2);

// host setup (bddc_host.cpp)
void host_assemble_upper(rawvec<int>& ia, rawvec<int>& ja, rawvec<double>& a);
void host_nodal_components(Subdomain& s);
void host_setup(Solver& S);              // everything integer/geometric + BC + weights + constraints
void host_interior_ordering(Subdomain& s, const vector<int>& f_ptr, const vector<int>& f_col,
                            const vector<double>& f_val);
void full_symmetric_csr(const Subdomain& s, vector<int>& ptr, vector<int>& col, vector<double>& val);
void host_prepare_blocks(Subdomain& s, SubBlocks& b);
// reduced-rhs inputs of a subdomain: weighted rhs with Dirichlet rows replaced by the
// weighted eliminated contributions; fo in the band order of the interior, fi per interface dof
void host_reduced_rhs_inputs(const Subdomain& s, vector<double>& fo, vector<double>& fi);
void host_reduced_rhs_inputs(const Subdomain& s, const double* rhs, bool complete, vector<double>& fo,
                             vector<double>& fi);
// new boundary values / loads after setup: recompute bc on every subdomain and
// assemble it over the interface (module_levels.f90:855-903)
void host_new_data(Solver& S);
// reactions A_fixed u - f on every subdomain, assembled on the interface
// (dd_compute_reactions, module_dd.f90:1258-1374)
void host_reactions(Solver& S);

// device (bddc_device.cu)
Device* device_create(Error& err);
Device* device_create_on_stream(Device* parent, Error& err);  // shares the parent's stream
bool device_release_memory(Error& err);
bool device_set_wait_limit(long long spins, Error& err);
bool device_new_data(Solver& S, Error& err);
// PCG on nrhs batched right-hand sides (Subdomain::rhs_batch) together; the
// solutions go to Subdomain::sol_batch, per-column results to the vectors
bool device_solve_batch(Solver& S, int nrhs, double tol, int maxit, int ndecrmax, vector<int>& num_iter,
                        vector<int>& reason, vector<double>& cond, Error& err);
bool device_element_gradient(int nelem, int nne, const int* inet, const double* ke0, bool per_element,
                             const double* u, const double* lam, double* grad, Error& err);
// largest subdomain interface the allocation-free dot product's fixed scratch holds
constexpr int NOALLOC_MAX_IFACE = 65536;
bool device_dotprod_noalloc(const int* iface_dofs, const double* weights, int nif, const double* v1,
                            const double* v2, int ndof, double* out, Error& err);
void device_destroy(Device* d);
bool device_setup(Solver& S, Error& err);
bool device_solve(Solver& S, int method, double tol, int maxit, int ndecrmax, int recycling, int maxvec, int& num_iter,
                  int& reason, double& cond,
                  Error& err);
bool device_download(Solver& S, int isub, double* out, Error& err);
void device_set_profiling(Device* d, bool on);
void device_get_profile(Device* d, double* ms, int* cnt);

double wall_time();

}  // namespace bddc
