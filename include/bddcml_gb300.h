/*
 * bddcml_gb300 -- GB300-native BDDC interface solver, C ABI.
 *
 * Drop-in replacement for the C interface of BDDCML (reference header
 * src/bddcml_interface_c.h).  Every entry point below has the signature of the
 * reference function it replaces: all arguments are pointers (Fortran
 * by-reference convention), int = c_int, double = c_double.  A Fortran caller
 * binds them through iso_c_binding exactly as the reference's
 * module_bddcml_c_wrapper.f90 does.
 *
 * Semantics follow the reference (module_bddcml.f90):
 *   - one global solver instance per process, not thread-safe, not re-entrant
 *     (module_levels.f90:158-175);
 *   - call order: init -> upload_subdomain_data (every subdomain) ->
 *     setup_preconditioner -> solve -> download_local_solution, optionally
 *     change_subdomain_data + setup_new_data + solve, then finalize;
 *   - numbase (0 for C, 1 for Fortran) shifts every index array and isub
 *     (module_levels.f90:249, 718);
 *   - inputs are copied; the caller keeps ownership of every array.
 *
 * Differences, all additive:
 *   - All subdomains live on one GPU in one process: comm_init/comm_all are
 *     accepted and ignored, nsub_loc_1 = -1 returns nsublev[0].
 *   - The reference aborts the process on errors (module_utils.f90:296-298).
 *     Here a failing call returns early and records a status that
 *     bddcml_get_last_error_c() reports; the process is not aborted.
 *   - There is no CPU fallback: without a usable CUDA device every call fails
 *     with status BDDCML_ERR_CUDA.
 */
#ifndef BDDCML_GB300_H
#define BDDCML_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define BDDCML_OK 0
#define BDDCML_ERR_ARGUMENT 1    /* bad size / index / order of calls          */
#define BDDCML_ERR_CUDA 2        /* CUDA runtime failure or no device          */
#define BDDCML_ERR_NUMERIC 3     /* non-positive pivot, NaN, singular coarse   */
#define BDDCML_ERR_UNSUPPORTED 4 /* feature outside the implemented scope      */
#define BDDCML_ERR_MEMORY 5      /* device or host allocation failed           */

/* ------------------------------------------------ reference entry points */

/* replaces bddcml_init_c, src/bddcml_interface_c.h:6-7 (module_bddcml.f90:36-101).
 * nl = 2 or 3; with three levels nsublev = {subdomains, level-2 subdomains, 1}
 * and the level-2 subdomains are formed by recursive coordinate bisection of
 * the level-1 subdomain centroids (the reference divides with METIS). */
void bddcml_init_c(int *nl, int *nsublev, int *lnsublev, int *nsub_loc_1, int *comm_init,
                   int *verbose_level, int *numbase, int *just_direct_solve_int);

/* replaces bddcml_upload_global_data_c, src/bddcml_interface_c.h:9-13.
 * Global loading is outside the implemented path: sets BDDCML_ERR_UNSUPPORTED. */
void bddcml_upload_global_data_c(int *nelem, int *nnod, int *ndof, int *ndim, int *meshdim,
                                 int *inet, int *linet, int *nnet, int *lnnet, int *nndf, int *lnndf,
                                 double *xyz, int *lxyz1, int *lxyz2,
                                 int *ifix, int *lifix, double *fixv, int *lfixv, double *rhs, int *lrhs,
                                 double *sol, int *lsol, int *idelm,
                                 int *neighbouring, int *load_division_int);

/* Global loading for C callers (extension).  The arguments of
 * bddcml_upload_global_data_c, except that the element matrices come from
 * the file named by elm_file instead of an open Fortran unit: a Fortran
 * unformatted sequential file (4-byte record markers) with one record
 * "lelm, elm(1:lelm)" per element in element order, each matrix packed as the
 * reference packs it (column by column, upper triangle for matrixtype 1/2,
 * full for 0; sm_pmd_make_element_numbering, module_sm.f90:272-380).  rhs is
 * the assembled global load.  At bddcml_setup_preconditioner_c the elements
 * are divided into nsublev[0] subdomains by recursive coordinate bisection of
 * their centroids (the reference uses METIS) and the data are localised;
 * everything after that is the subdomain path.  load_division_int must be 0. */
void bddcml_upload_global_data_file_c(int *nelem, int *nnod, int *ndof, int *ndim, int *meshdim,
                                      int *inet, int *linet, int *nnet, int *lnnet, int *nndf, int *lnndf,
                                      double *xyz, int *lxyz1, int *lxyz2,
                                      int *ifix, int *lifix, double *fixv, int *lfixv,
                                      double *rhs, int *lrhs, double *sol, int *lsol, const char *elm_file,
                                      int *neighbouring, int *load_division_int);

/* replaces bddcml_upload_subdomain_data_c, src/bddcml_interface_c.h:15-27
 * (module_bddcml.f90:186-356, module_levels.f90:615-782).  matrixtype 1 (SPD)
 * and 2 (symmetric) take the upper triangle; 0 (general) takes all entries and
 * is solved with LU factors and a dual coarse basis (use BiCGSTAB, method 1);
 * three levels, adaptive constraints, batched loads and reactions need a
 * symmetric matrix (BDDCML_ERR_UNSUPPORTED otherwise).  Indices are checked
 * after the numbase shift: INET within [0, nnods), ISNGN / ISVGVN / ISEGN not
 * negative, both matrix indices within [0, ndofs), and row <= column for
 * matrixtype 1 and 2.  A failed check sets BDDCML_ERR_ARGUMENT and leaves the
 * subdomain not loaded, so the call can be repeated with corrected data. */
void bddcml_upload_subdomain_data_c(int *nelem, int *nnod, int *ndof, int *ndim, int *meshdim,
                                    int *isub, int *nelems, int *nnods, int *ndofs,
                                    int *inet, int *linet, int *nnet, int *lnnet, int *nndf, int *lnndf,
                                    int *isngn, int *lisngn, int *isvgvn, int *lisvgvn, int *isegn, int *lisegn,
                                    double *xyz, int *lxyz1, int *lxyz2,
                                    int *ifix, int *lifix, double *fixv, int *lfixv,
                                    double *rhs, int *lrhs, int *is_rhs_complete,
                                    double *sol, int *lsol,
                                    int *matrixtype, int *i_sparse, int *j_sparse, double *a_sparse, int *la,
                                    int *is_assembled_int,
                                    double *user_constraints, int *luser_constraints1, int *luser_constraints2,
                                    double *element_data, int *lelement_data1, int *lelement_data2,
                                    double *dof_data, int *ldof_data,
                                    int *find_components_int, int *use_dual_mesh_graph_int, int *neighbouring);

/* replaces bddcml_setup_preconditioner_c, src/bddcml_interface_c.h:29-35
 * (module_bddcml.f90:359-455, module_levels.f90:905-1069) */
void bddcml_setup_preconditioner_c(int *matrixtype, int *use_defaults_int, int *parallel_division_int,
                                   int *use_corner_constraints_int, int *use_arithmetic_constraints_int,
                                   int *use_adaptive_constraints_int, int *use_user_constraints_int,
                                   int *weights_type);

/* replaces bddcml_solve_c, src/bddcml_interface_c.h:37-39 (module_bddcml.f90:459-567).
 * method 0 PCG (with the Lanczos condition estimate), 1 BiCGSTAB, 2 steepest
 * descent; -1 takes the reference defaults (module_bddcml.f90:515-520):
 * BiCGSTAB, tol 1e-6, maxit 1000, ndecrmax 30, ignoring the passed values.
 * condition_number is -1 for methods 1 and 2.  With method 0, recycling_int = 1
 * keeps up to max_number_of_stored_vectors S-orthonormal search directions
 * across solves (module_krylov.f90:313-484, 663-726): they project the initial
 * residual of the next solve (after bddcml_setup_new_data_c) and every new
 * direction is orthogonalised against them; the capacity is fixed by the first
 * recycling solve and the basis is dropped at the next setup or at finalize.
 * method 5 (direct solve) sets
 * BDDCML_ERR_UNSUPPORTED, any other value BDDCML_ERR_ARGUMENT.  A steepest
 * descent that stalls for ndecrmax iterations sets BDDCML_ERR_NUMERIC (the
 * reference stops with an error there, module_krylov.f90:1801-1812). */
void bddcml_solve_c(int *comm_all, int *method, double *tol, int *maxit, int *ndecrmax,
                    int *recycling_int, int *max_number_of_stored_vectors,
                    int *num_iter, int *converged_reason, double *condition_number);

/* replaces bddcml_download_local_solution_c, src/bddcml_interface_c.h:41 */
void bddcml_download_local_solution_c(int *isub, double *sols, int *lsols);

/* Batched loads (extension; the reference solves one load per bddcml_solve_c
 * call and re-enters with change_subdomain_data + setup_new_data for the next).
 * Uploads nrhs (1..64) right-hand sides of subdomain isub, rhss holding nrhs
 * columns of ndof entries (column-major, *lrhss = ndof * nrhs); the fixed
 * values, matrix and constraints are those of the set-up problem. */
void bddcml_upload_subdomain_rhs_batch_c(int *isub, int *nrhs, double *rhss, int *lrhss, int *is_rhs_complete);

/* Solves the uploaded batch by PCG (method 0; any other method sets
 * BDDCML_ERR_UNSUPPORTED).  Every column runs the iteration of
 * bddcml_solve_c with its own scalars and stop test (module_krylov.f90:545-888)
 * from the zero initial guess (fixed values at fixed dofs); the subdomain
 * applies of all columns run as one product per subdomain.  num_iter,
 * converged_reason and condition_number receive nrhs entries each. */
void bddcml_solve_batch_c(int *comm_all, int *method, double *tol, int *maxit, int *ndecrmax, int *nrhs,
                          int *num_iter, int *converged_reason, double *condition_number);

/* Products of the batched solve in mixed precision.  Mode 1 slices S and every
 * block of search directions into 6-bit integer pieces and multiplies them on
 * the bf16 tensor cores with exact accumulation of the leading terms
 * (FP64-class products; used when every subdomain has at most 3264 interface
 * dofs, else mode 0), and runs the FP32 preconditioner products as 3xTF32 on
 * the tensor cores.  Mode 2 also slices the FP32 preconditioner blocks (Z, Phi,
 * Phi^T) and their FP64 operands, so that every preconditioner application is
 * the same linear operator without rounding noise (which costs outer
 * iterations on ill-conditioned problems).  Mode 0 multiplies the FP32 (hi, lo)
 * pairs of S in double-float arithmetic and the preconditioner blocks in FP32
 * on the FP32 pipes.  Mode -1 (the default) takes 2 when the setup's interior
 * solves needed more than the two standard refinement steps (stiff
 * subdomains) and 1 otherwise.  Takes effect at the next bddcml_solve_batch_c.
 * No counterpart in the reference. */
void bddcml_set_batch_operator_c(int *mode);

/* Solutions of the last batched solve for subdomain isub: nrhs columns of ndof
 * entries, column-major (*lsols = ndof * nrhs). */
void bddcml_download_local_solution_batch_c(int *isub, int *nrhs, double *sols, int *lsols);

/* replaces bddcml_download_global_solution_c, src/bddcml_interface_c.h:43
 * (module_levels.f90:4617-4744): every subdomain's solution written at its
 * global dofs; *lsol must be the global dof count. */
void bddcml_download_global_solution_c(double *sol, int *lsol);

/* replaces bddcml_download_local_reactions_c, src/bddcml_interface_c.h:45
 * (module_dd.f90:1258-1374, 3364-3395): A_fixed u - f of the subdomain after a
 * solve, A_fixed the uploaded entries in fixed rows and columns, values on
 * shared dofs summed over the subdomains, the load subtracted on fixed dofs. */
void bddcml_download_local_reactions_c(int *isub, double *reas, int *lreas);

/* replaces bddcml_download_global_reactions_c, src/bddcml_interface_c.h:47
 * (module_levels.f90:4785-4914): the subdomains' reactions at their global dofs. */
void bddcml_download_global_reactions_c(double *rea, int *lrea);

/* replaces bddcml_change_global_data_c, src/bddcml_interface_c.h:49: new fixed
 * values, loads and initial guess of data loaded by
 * bddcml_upload_global_data_file_c (BDDCML_ERR_UNSUPPORTED otherwise), after
 * setup and with the same fixed dofs; takes effect at bddcml_setup_new_data_c. */
void bddcml_change_global_data_c(int *ifix, int *lifix, double *fixv, int *lfixv, double *rhs, int *lrhs,
                                 double *sol, int *lsol);

/* replaces bddcml_change_subdomain_data_c, src/bddcml_interface_c.h:51-54
 * (module_levels.f90:785-849).  New fixed values, loads and initial guess of a
 * subdomain after setup; the set of fixed dofs must stay the same
 * (BDDCML_ERR_UNSUPPORTED otherwise, since the eliminated matrix and the
 * coarse space depend on it).  Takes effect at bddcml_setup_new_data_c. */
void bddcml_change_subdomain_data_c(int *isub, int *ifix, int *lifix, double *fixv, int *lfixv,
                                    double *rhs, int *lrhs, int *is_rhs_complete, double *sol, int *lsol);

/* replaces bddcml_setup_new_data_c, src/bddcml_interface_c.h:56 (module_levels.f90:852-903).
 * Recomputes the eliminated Dirichlet contributions and the reduced
 * right-hand side with the factors, Schur complements and preconditioner of
 * the last setup; the next bddcml_solve_c solves the new problem. */
void bddcml_setup_new_data_c(void);

/* replaces bddcml_dotprod_subdomain_c, src/bddcml_interface_c.h:58 (module_dd.f90:12736-12788) */
void bddcml_dotprod_subdomain_c(int *isub, double *vec1, int *lvec1, double *vec2, int *lvec2, double *dotprod);

/* replaces bddcml_finalize_c, src/bddcml_interface_c.h:60 */
void bddcml_finalize_c(void);

/* ------------------------------------------------------------ extensions */

/* Status of the last call (BDDCML_OK ... BDDCML_ERR_MEMORY); copies a
 * NUL-terminated message into msg (at most *lmsg bytes, may be NULL).  The
 * reference aborts instead (module_utils.f90:265-298); this has no
 * counterpart there. */
int bddcml_get_last_error_c(char *msg, int *lmsg);

/* Arithmetic of the subdomain factors, Schur-complement preconditioner blocks
 * and coarse basis: 0 = plain FP64 everywhere, 1 = mixed (FP32 factors and
 * preconditioner blocks with FP64 refinement of the Schur operator; FP64 PCG
 * vectors, dot products, weights and coarse solve).  Default 1.  Must be set
 * before bddcml_setup_preconditioner_c.  No counterpart in the reference. */
void bddcml_set_precision_c(int *mode);

/* Timing and size report of the last setup and solve, filled into stats
 * (length *lstats, up to 64 doubles; see bddcml_gb300/__init__.py for the
 * field list).  No counterpart in the reference. */
void bddcml_get_stats_c(double *stats, int *lstats);

/* Relative residual history of the last PCG solve (at most *lhist values);
 * *lhist returns the number of iterations recorded.  Corresponds to the
 * per-iteration residual print of module_krylov.f90:769-772. */
void bddcml_get_residual_history_c(double *hist, int *lhist);

/* Copies the interface weights of subdomain *isub (ndofi values, subdomain
 * interface order) for checking; no counterpart in the reference. */
void bddcml_get_interface_weights_c(int *isub, double *wi, int *lwi);

/* Structural summary of the coarse space: out = {ncorner, nedge, nface,
 * ndofc, sum ndofi, sum ndofo}.  Corresponds to the level summary of
 * module_levels.f90:2240-2300 (printed there, returned here). */
void bddcml_get_coarse_info_c(int *out, int *lout);

/* 64-bit digest (FNV-1a) of every host-side setup result: the assembled
 * subdomain matrices, mesh components, interface and interior dof lists,
 * coarse nodes and constraint rows, eliminated Dirichlet values, weights,
 * unique interface numbering and interior orderings.  The host setup runs on
 * all host threads with fixed orders of work, so the digest does not depend
 * on the thread count.  Available after the host part of
 * bddcml_setup_preconditioner_c.  No counterpart in the reference. */
void bddcml_get_setup_digest_c(unsigned long long *digest);

/* Switches the per-phase CUDA-event timers on (1) or off (0).  The two totals
 * (numeric setup, solve) are always timed.  No counterpart in the reference
 * (its verbosity-2 profiling prints wall times, module_bddcml.f90:91-93). */
void bddcml_set_profiling_c(int *on);

/* Accumulated milliseconds and counts per timed phase since the last
 * setup_preconditioner (see bddcml_gb300/__init__.py PHASES for the order);
 * *lphase in: capacity, out: number of phases. */
void bddcml_get_profile_c(double *ms, int *counts, int *lphase);

/* Device memory of a solver is taken from a per-process CUDA memory pool
 * that keeps freed memory for the next setup (bddcml_finalize_c returns the
 * solver's memory to that pool, not to the driver).  This call hands all
 * unused pooled memory back to the driver; it may be called at any time.
 * No counterpart in the reference. */
void bddcml_release_device_memory_c(void);

/* Spin limit of every wait inside the tensor-core sweep kernels of the
 * current device (*spins <= 0 restores the default, 2^26 polls).  A wait that
 * runs out stops its kernel cleanly (bulk copies and MMAs in flight are
 * drained, tensor memory is freed) and the setup fails with
 * BDDCML_ERR_NUMERIC; the next setup starts clean.  Meant for testing that
 * path with a tiny limit.  No counterpart in the reference, whose errors
 * abort (module_utils.f90:296-298). */
void bddcml_set_wait_limit_c(long long *spins);

/* Eigenvalue threshold tau of the adaptive face constraints (no counterpart in
 * the reference, which fixes it at 1.5: threshold_eigval_default,
 * module_adaptivity.f90:30).  Eigenvectors of the face-pair problems with
 * eigenvalue >= tau become constraints.  Takes effect at the next
 * bddcml_setup_preconditioner_c; tau must be positive (BDDCML_ERR_ARGUMENT). */
void bddcml_set_adaptive_threshold_c(double *tau);

/* Face pairs of the last adaptive setup (no counterpart in the reference):
 * for p < min(*lpair, npair), pairs[3p..3p+2] = the two subdomains (numbase
 * applied) and the number of computed eigenvalues k, eigs[10p..10p+9] the
 * eigenvalues in descending order (zero beyond k).  *lpair returns npair. */
void bddcml_get_adaptive_info_c(int *pairs, double *eigs, int *lpair);

/* Per-element gradient of an objective J(u) with respect to element
 * coefficients kappa_e, for K(kappa) = sum_e kappa_e K_e^0:
 *     grad[e] = dJ/dkappa_e = - lambda_e^T K_e^0 u_e,
 * where u is the solution and lambda the adjoint solution (K lambda = dJ/du
 * with homogeneous Dirichlet values, e.g. from change_subdomain_data +
 * setup_new_data + solve).  All arrays are device pointers: inet (nelem x nne
 * global dof indices, 0-based), ke0 (one nne x nne row-major matrix, or one
 * per element when *ke0_per_element != 0), u and lam (global vectors), grad
 * (nelem).  nne <= 27.  Runs on the legacy default stream and waits for it.
 * No counterpart in the reference. */
void bddcml_element_gradient_dev_c(int *nelem, int *nne, const int *inet, const double *ke0,
                                   int *ke0_per_element, const double *u, const double *lam, double *grad);

/* The weighted dot product of bddcml_dotprod_subdomain_c for vectors that
 * already live in device memory (vec1, vec2: device pointers, length *lvec =
 * the subdomain's ndof, subdomain dof order); the result is written to the
 * host double *dotprod.  No counterpart in the reference.
 *
 * It allocates nothing, on the device or through any library: its scratch
 * (the subdomain's interface weights and indices, block partial sums, the
 * result) is one fixed array in static device memory of about 0.8 MB, which
 * every GPU that loads the library keeps until the process exits.  It holds
 * subdomains with at most 65536 interface dofs; a larger interface is
 * rejected with BDDCML_ERR_ARGUMENT.  The array keeps the previous call's
 * contents; the one counter that must start at zero is cleared by each call
 * before its kernel runs.  It is meant for callers that keep their
 * vectors on the GPU and may not allocate at that point: an application that
 * reserves all device memory up front, or one whose own allocator forbids
 * device allocations (and the implicit device synchronisation of cudaMalloc
 * and cudaFree) inside its time-stepping loop.
 *
 * The first call on each device looks up the scratch address
 * (cudaGetSymbolAddress).  Under CUDA's lazy module loading (the default since
 * CUDA 12.2) that first call also loads the library's module on the device,
 * which is when the static array is placed in device memory: make one call per
 * device before any region where allocation is not allowed, and before any
 * stream capture.  Later calls allocate nothing.  Work
 * runs on the legacy default stream; the vectors must be ready there.  Calls
 * must not overlap in time (several host threads, several streams): they share
 * the scratch and would race.  Needs a finished bddcml_setup_preconditioner_c. */
void bddcml_dotprod_subdomain_dev_c(int *isub, const double *vec1, const double *vec2, int *lvec,
                                    double *dotprod);

#ifdef __cplusplus
}
#endif

#endif /* BDDCML_GB300_H */
