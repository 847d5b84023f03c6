/* A C caller of the BDDC interface, written against the reference's C API
 * (src/bddcml_interface_c.h:6-60 of sistek/bddcml) and nothing else: the
 * header is chosen at compile time (-DBDDCML_HEADER=...), so the same source
 * compiles against the reference's unmodified header and against
 * include/bddcml_gb300.h.  Test infrastructure.
 *
 *   abi_driver <problem file> <solution file>
 *
 * The problem file (written by tests/test_abi_driver.py) holds, as 32-bit
 * ints and 64-bit doubles in native order:
 *   nelem nnod ndof ndim meshdim nsub matrixtype, then tol
 *   per subdomain: isub nelems nnods ndofs linet la is_rhs_complete,
 *     inet[linet] nnet[nelems] nndf[nnods] isngn[nnods] isvgvn[ndofs]
 *     isegn[nelems] xyz[nnods*ndim] (column-major) ifix[ndofs] fixv[ndofs]
 *     rhs[ndofs] sol[ndofs] i_sparse[la] j_sparse[la] a_sparse[la]
 * The call sequence is the one of the reference example
 * (examples/poisson_on_cube.f90:373-672): init, upload every subdomain,
 * setup, PCG solve, download every subdomain's solution, finalize.  The
 * solution file receives num_iter, converged_reason, condition_number and
 * each subdomain's ndofs values. */
#include <stdio.h>
#include <stdlib.h>

#include BDDCML_HEADER

static FILE* in;

static int read_int(void) {
  int v;
  if (fread(&v, sizeof v, 1, in) != 1) { fprintf(stderr, "short read\n"); exit(2); }
  return v;
}

static void* read_arr(size_t n, size_t sz) {
  void* p = malloc(n ? n * sz : 1);
  if (!p || fread(p, sz, n, in) != n) { fprintf(stderr, "short read\n"); exit(2); }
  return p;
}

int main(int argc, char** argv) {
  if (argc != 3) { fprintf(stderr, "usage: abi_driver problem solution\n"); return 2; }
  in = fopen(argv[1], "rb");
  if (!in) { perror(argv[1]); return 2; }
  int nelem = read_int(), nnod = read_int(), ndof = read_int(), ndim = read_int(), meshdim = read_int();
  int nsub = read_int(), matrixtype = read_int();
  double tol;
  if (fread(&tol, sizeof tol, 1, in) != 1) return 2;

  int nl = 2, nsublev[2] = {nsub, 1}, lnsublev = 2, nsub_loc_1 = -1, comm = 0, verbose = 0, numbase = 0, direct = 0;
  bddcml_init_c(&nl, nsublev, &lnsublev, &nsub_loc_1, &comm, &verbose, &numbase, &direct);

  int* sub_ndofs = malloc(sizeof(int) * nsub);
  int* sub_isub = malloc(sizeof(int) * nsub);
  for (int t = 0; t < nsub; ++t) {
    int isub = read_int(), nelems = read_int(), nnods = read_int(), ndofs = read_int(), linet = read_int();
    int la = read_int(), is_rhs_complete = read_int();
    int* inet = read_arr(linet, sizeof(int));
    int* nnet = read_arr(nelems, sizeof(int));
    int* nndf = read_arr(nnods, sizeof(int));
    int* isngn = read_arr(nnods, sizeof(int));
    int* isvgvn = read_arr(ndofs, sizeof(int));
    int* isegn = read_arr(nelems, sizeof(int));
    double* xyz = read_arr((size_t)nnods * ndim, sizeof(double));
    int* ifix = read_arr(ndofs, sizeof(int));
    double* fixv = read_arr(ndofs, sizeof(double));
    double* rhs = read_arr(ndofs, sizeof(double));
    double* sol = read_arr(ndofs, sizeof(double));
    int* isp = read_arr(la, sizeof(int));
    int* jsp = read_arr(la, sizeof(int));
    double* asp = read_arr(la, sizeof(double));
    int lnnet = nelems, lnndf = nnods, lisngn = nnods, lisvgvn = ndofs, lisegn = nelems, lxyz1 = nnods,
        lxyz2 = ndim, lifix = ndofs, lfixv = ndofs, lrhs = ndofs, lsol = ndofs, is_assembled = 0;
    double user_constraints[1] = {0.0}, element_data[1] = {0.0}, dof_data[1] = {0.0};
    int zero = 0, find_components = 1, use_dual_mesh_graph = 1, neighbouring = 3;
    bddcml_upload_subdomain_data_c(&nelem, &nnod, &ndof, &ndim, &meshdim, &isub, &nelems, &nnods, &ndofs, inet,
                                   &linet, nnet, &lnnet, nndf, &lnndf, isngn, &lisngn, isvgvn, &lisvgvn, isegn,
                                   &lisegn, xyz, &lxyz1, &lxyz2, ifix, &lifix, fixv, &lfixv, rhs, &lrhs,
                                   &is_rhs_complete, sol, &lsol, &matrixtype, isp, jsp, asp, &la, &is_assembled,
                                   user_constraints, &zero, &zero, element_data, &zero, &zero, dof_data, &zero,
                                   &find_components, &use_dual_mesh_graph, &neighbouring);
    sub_ndofs[t] = ndofs;
    sub_isub[t] = isub;
    free(inet); free(nnet); free(nndf); free(isngn); free(isvgvn); free(isegn); free(xyz);
    free(ifix); free(fixv); free(rhs); free(sol); free(isp); free(jsp); free(asp);
  }
  fclose(in);

  int use_defaults = 0, parallel_division = 1, corners = 1, arithmetic = 1, adaptive = 0, user = 0, weights = 0;
  bddcml_setup_preconditioner_c(&matrixtype, &use_defaults, &parallel_division, &corners, &arithmetic, &adaptive,
                                &user, &weights);
  int method = 0, maxit = 500, ndecrmax = 50, recycling = 0, maxvec = 0, num_iter = 0, reason = -99;
  double cond = 0.0;
  bddcml_solve_c(&comm, &method, &tol, &maxit, &ndecrmax, &recycling, &maxvec, &num_iter, &reason, &cond);

  FILE* out = fopen(argv[2], "wb");
  if (!out) { perror(argv[2]); return 2; }
  fwrite(&num_iter, sizeof num_iter, 1, out);
  fwrite(&reason, sizeof reason, 1, out);
  fwrite(&cond, sizeof cond, 1, out);
  for (int t = 0; t < nsub; ++t) {
    double* sols = malloc(sizeof(double) * (sub_ndofs[t] ? sub_ndofs[t] : 1));
    int isub = sub_isub[t], lsols = sub_ndofs[t];
    bddcml_download_local_solution_c(&isub, sols, &lsols);
    fwrite(sols, sizeof(double), (size_t)lsols, out);
    free(sols);
  }
  fclose(out);
  bddcml_finalize_c();
  free(sub_ndofs);
  free(sub_isub);
  return 0;
}
