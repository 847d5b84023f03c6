// Batched interface PCG: nrhs right-hand sides of one set-up problem solved
// together (an extension of bddcml_solve; the reference solves one load per
// call, module_bddcml.f90:505-600).  Every column runs the PCG of
// module_krylov.f90:545-888 with its own scalars and stop test; the
// subdomain applies of all columns are GEMMs (bddc_batch_kernels.cuh), so each
// Schur complement, local preconditioner block and interior-resolve block is
// read once per iteration for the whole batch.
//
// Included by bddc_device.cu after the Device class, whose buffers, setup
// results and single-column routines (reduced_rhs_device, run_solve) it uses.

namespace bddc {

static unsigned blocks_for(long long cnt, int threads = 256) { return (unsigned)((cnt + threads - 1) / threads); }

// Launch-shape autotuner: for a key (kernel, device, problem sizes, batch
// width) it times every candidate with CUDA events on the library stream (one
// warm-up launch, then three timed launches) and keeps the fastest for the
// rest of the process.  The candidates must all be valid launches.
static int tune_pick(Device& D, const std::string& key, const vector<int>& cands,
                     const std::function<void(int)>& run, float* best_ms = nullptr) {
  static std::mutex mu;
  static std::map<std::string, std::pair<int, float>> cache;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  const std::string k = std::to_string(dev) + ":" + key;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(k);
    if (it != cache.end()) {
      if (best_ms) *best_ms = it->second.second;
      return it->second.first;
    }
  }
  int pick = cands.empty() ? 0 : cands[0];
  float best = 0.f;
  if (cands.size() > 1) {
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    best = 1e30f;
    for (int c : cands) {
      run(c);
      CK(cudaEventRecord(e0, D.st));
      for (int r = 0; r < 3; ++r) run(c);
      CK(cudaEventRecord(e1, D.st));
      CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) { best = ms; pick = c; }
    }
    CK(cudaEventDestroy(e0));
    CK(cudaEventDestroy(e1));
    best /= 3.f;
  }
  std::lock_guard<std::mutex> lk(mu);
  cache[k] = {pick, best};
  if (best_ms) *best_ms = best;
  return pick;
}

// K-split candidates of a product whose job list has ntile row tiles with at
// least minch K chunks each: 1, 2, 4, 8 parts, none with an empty part
static vector<int> ksplit_candidates(int minch) {
  vector<int> c;
  for (int ks = 1; ks <= 8; ks *= 2)
    if (ks == 1 || ks <= minch) c.push_back(ks);
  return c;
}

// out = addend + [A1 A2] [B1; B2] for every descriptor (kb_gemm_t), rows up to maxm
template <typename T>
static void gemm_t(Device& D, const GemmDesc* gd, int ndesc, int maxm, const T* A, const T* B1, const T* B2, int ldb,
                   double* out, const double* addend, int ldo, int nk, const int* ndone) {
  const size_t smem = GtCfg<T>::SMEM;
  raise_smem(kb_gemm_t<T>, smem);
  kb_gemm_t<T><<<dim3((maxm + GtCfg<T>::BM - 1) / GtCfg<T>::BM, ndesc), 256, smem, D.st>>>(gd, A, B1, B2, ldb, out,
                                                                                          addend, ldo, nk, ndone);
  CKL();
}

// Slices of the Schur complements for the tensor-core apply (bddc_ozaki.cuh),
// made once per batch setup from the float2 operator.
static void batch_prepare_oz(Device& D) {
  BatchBufs& B = D.bt;
  auto& mem = B.mem;
  vector<long long> soff(D.nsub), eoff(D.nsub), xoff(D.nsub);
  long long ns = 0, ne = 0, nx = 0;
  int maxrt = 0, maxch = 0;
  for (int t = 0; t < D.nsub; ++t) {
    const int ni = D.hs[t].ni;
    const int nrt = (ni + OZ_M - 1) / OZ_M, nch = (ni + OZ_KC - 1) / OZ_KC;
    soff[t] = ns; ns += (long long)nrt * nch * OZ_NS * OZ_AB;
    eoff[t] = ne; ne += (long long)nrt * OZ_M;
    xoff[t] = nx; nx += (long long)nch * OZ_BB;
    maxrt = std::max(maxrt, nrt);
    maxch = std::max(maxch, nch);
  }
  B.oz_nrt = maxrt;
  B.oz_nch = maxch;
  B.oz_s = dalloc<__nv_bfloat16>(std::max(1LL, ns), mem);
  B.oz_x = dalloc<__nv_bfloat16>(std::max(1LL, nx), mem);
  B.oz_erow = dalloc<int>(std::max(1LL, ne), mem);
  B.oz_fcol = dalloc<int>((long long)D.nsub * BMAX, mem);
  B.oz_soff = upload(soff, mem, D.st);
  B.oz_eoff = upload(eoff, mem, D.st);
  B.oz_xoff = upload(xoff, mem, D.st);
  const float2* S = static_cast<const float2*>(D.poolS);
  kb_oz_row_exp<<<dim3((maxrt * OZ_M + 7) / 8, D.nsub), 256, 0, D.st>>>(D.ds, S, B.oz_eoff, B.oz_erow);
  CKL();
  kb_oz_slice_s<<<dim3(maxrt * maxch, D.nsub), 256, 0, D.st>>>(D.ds, S, B.oz_soff, B.oz_eoff, B.oz_erow, B.oz_s);
  CKL();
  B.oz = true;
}

// A tiles and job lists of the 3xTF32 preconditioner products (bddc_batch_tc.cuh),
// made once per batch setup: [Z | Phi] from the preconditioner pool, Phi^T from phit
static void batch_prepare_tc(Device& D) {
  BatchBufs& B = D.bt;
  auto& mem = B.mem;
  const bool coarse = D.ndofc > 0;
  int dev = 0, nsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  B.tc_grid = std::max(1, nsm);
  // the Phi^T product has one tile per subdomain: its K range is split into
  // parts (each writing its own plane of tc_rcs) so that the job list fills the
  // SMs; the number of parts is picked by the autotuner below
  long long ncon = 0;
  int minch = 1 << 30;
  for (auto& d : D.hs) {
    ncon = std::max(ncon, (long long)d.coff + d.nc);
    if (coarse && d.nc > 0) minch = std::min(minch, (d.ni + TC_KC - 1) / TC_KC);
  }
  vector<long long> zoff(D.nsub), poff(D.nsub), boff(D.nsub);
  vector<TcJob> jz;
  long long nz = 0, np = 0, nb = 0;
  int mch1 = 0, mch2 = 0, maxz = 0, maxp = 0;
  for (int t = 0; t < D.nsub; ++t) {
    const DevSub& d = D.hs[t];
    const int n1 = (d.ni + TC_KC - 1) / TC_KC, n2 = coarse ? (d.nc + TC_KC - 1) / TC_KC : 0;
    mch1 = std::max(mch1, n1);
    mch2 = std::max(mch2, n2);
    boff[t] = nb;
    nb += (long long)(n1 + n2) * GC_TILE;
    const int nrz = (d.ni + TC_M - 1) / TC_M;
    zoff[t] = nz;
    for (int rt = 0; rt < nrz; ++rt)
      jz.push_back(TcJob{nz + (long long)rt * (n1 + n2) * GC_TILE, boff[t], (long long)d.rep + rt * TC_M,
                         std::min(TC_M, d.ni - rt * TC_M), n1 + n2});
    nz += (long long)nrz * (n1 + n2) * GC_TILE;
    maxz = std::max(maxz, nrz * (n1 + n2));
    const int nrp = coarse ? (d.nc + TC_M - 1) / TC_M : 0;
    poff[t] = np;
    np += (long long)nrp * n1 * GC_TILE;
    maxp = std::max(maxp, nrp * n1);
  }
  auto make_jp = [&](int ks) {
    vector<TcJob> jp;
    for (int t = 0; t < D.nsub && coarse; ++t) {
      const DevSub& d = D.hs[t];
      const int n1 = (d.ni + TC_KC - 1) / TC_KC, nrp = (d.nc + TC_M - 1) / TC_M;
      for (int rt = 0; rt < nrp; ++rt)
        for (int h = 0; h < ks; ++h) {  // part h: chunks [c0, c1), rows in plane h
          const int c0 = (int)((long long)n1 * h / ks), c1 = (int)((long long)n1 * (h + 1) / ks);
          if (c1 > c0)
            jp.push_back(TcJob{poff[t] + ((long long)rt * n1 + c0) * GC_TILE, boff[t] + (long long)c0 * GC_TILE,
                               h * ncon + d.coff + rt * TC_M, std::min(TC_M, d.nc - rt * TC_M), c1 - c0});
        }
    }
    return jp;
  };
  B.tc_az = dalloc<float>(std::max(1LL, nz), mem);
  B.tc_ap = dalloc<float>(std::max(1LL, np), mem);
  B.tc_b = dalloc<float>(std::max(1LL, nb), mem);
  B.tc_boff = upload(boff, mem, D.st);
  B.tc_jz = upload(jz, mem, D.st);
  B.tc_njz = (int)jz.size();
  B.tc_mch1 = mch1;
  B.tc_mch2 = mch2;
  B.tc_pstride = std::max(1LL, ncon) * B.nk;
  B.tc_rcs = dalloc<double>(8 * B.tc_pstride, mem);  // room for the largest K split
  if (maxz > 0) {
    kb_tile_a<<<dim3(maxz, D.nsub), 256, 0, D.st>>>(B.gZ, upload(zoff, mem, D.st),
                                                     static_cast<const float*>(D.poolPC), B.tc_az);
    CKL();
  }
  if (coarse && maxp > 0) {
    kb_tile_a<<<dim3(maxp, D.nsub), 256, 0, D.st>>>(B.gP, upload(poff, mem, D.st),
                                                     static_cast<const float*>(B.phit), B.tc_ap);
    CKL();
  }
  // K split of the Phi^T product, timed on this batch's shapes
  int ks = 1;
  vector<TcJob> jp = make_jp(1);
  if (coarse && !jp.empty()) {
    vector<int> cands = ksplit_candidates(minch);
    vector<TcJob*> lists(9, nullptr);
    vector<int> counts(9, 0);
    for (int c : cands) {
      vector<TcJob> v = make_jp(c);
      lists[c] = upload(v, mem, D.st);
      counts[c] = (int)v.size();
    }
    const std::string key = "phit_tc3:" + std::to_string(D.nsub) + ":" + std::to_string(D.maxNI) + ":" +
                            std::to_string(D.ncpmax) + ":" + std::to_string(B.nk);
    raise_smem(kb_gemm_tc3, GC_SMEM);
    ks = tune_pick(D, key, cands, [&](int c) {
      kb_gemm_tc3<<<std::min(counts[c], B.tc_grid), GC_THREADS, GC_SMEM, D.st>>>(
          lists[c], counts[c], B.tc_ap, B.tc_b, B.tc_rcs, B.nk, B.nk, D.err, nullptr);
      CKL();
    });
    B.tc_jp = lists[ks];
    B.tc_njp = counts[ks];
  }
  B.tc_ks = ks;
  // planes that no job writes stay zero (the timing runs wrote into all of them)
  CK(cudaMemsetAsync(B.tc_rcs, 0, (size_t)8 * B.tc_pstride * sizeof(double), D.st));
}

// Sliced preconditioner blocks for exact products (bddc_ozaki.cuh), made once
// per batch setup: Z and Phi from the preconditioner pool, Phi^T from phit
// (offsets opt), with their job lists.  The application reuses the Schur
// apply's X slice buffers for w .* r and slices the coarse solution into ozp_u.
static void batch_prepare_ozpc(Device& D, const vector<long long>& opt) {
  BatchBufs& B = D.bt;
  auto& mem = B.mem;
  const int nsub = D.nsub;
  const bool coarse = D.ndofc > 0;
  auto nchk = [](int k) { return (k + OZ_KC - 1) / OZ_KC; };
  auto ntile = [](int m) { return (m + OZ_M - 1) / OZ_M; };
  const long long blk = (long long)OZ_NA * OZ_AB;  // bf16 elements of one sliced 128 x 64 chunk
  vector<OzMat> mpc, mpt;                          // from the preconditioner pool / from phit
  vector<long long> sz(nsub, 0), sphi(nsub, 0), spt(nsub, 0), ez(nsub, 0), ephi(nsub, 0), ept(nsub, 0);
  vector<long long> xo(nsub, 0), uo(nsub, 0);
  long long ns = 0, ne = 0, nx = 0, nu = 0, ncon = 0;
  int nchu = 0, blk_pc = 0, rows_pc = 0, blk_pt = 0, rows_pt = 0;
  for (int t = 0; t < nsub; ++t) {
    const DevSub& d = D.hs[t];
    ncon = std::max(ncon, (long long)d.coff + d.nc);
    xo[t] = nx;  // the layout of the Schur apply's X slices (batch_prepare_oz)
    nx += (long long)nchk(d.ni) * OZ_BB;
    const int nc = coarse ? d.nc : 0;
    uo[t] = nu;
    nu += (long long)nchk(nc) * OZ_BB;
    nchu = std::max(nchu, nchk(nc));
    sz[t] = ns;
    ns += (long long)ntile(d.ni) * nchk(d.ni) * blk;
    ez[t] = ne;
    ne += (long long)ntile(d.ni) * OZ_M;
    mpc.push_back(OzMat{d.oZ, sz[t], ez[t], d.NI, d.ni, d.ni});
    blk_pc = std::max(blk_pc, ntile(d.ni) * nchk(d.ni));
    rows_pc = std::max(rows_pc, ntile(d.ni) * OZ_M);
    if (nc > 0 && d.ni > 0) {
      sphi[t] = ns;
      ns += (long long)ntile(d.ni) * nchk(nc) * blk;
      ephi[t] = ne;
      ne += (long long)ntile(d.ni) * OZ_M;
      mpc.push_back(OzMat{d.oPhi, sphi[t], ephi[t], d.ncp, d.ni, nc});
      spt[t] = ns;
      ns += (long long)ntile(nc) * nchk(d.ni) * blk;
      ept[t] = ne;
      ne += (long long)ntile(nc) * OZ_M;
      mpt.push_back(OzMat{opt[t], spt[t], ept[t], d.NI, nc, d.ni});
      blk_pt = std::max(blk_pt, ntile(nc) * nchk(d.ni));
      rows_pt = std::max(rows_pt, ntile(nc) * OZ_M);
    }
  }
  B.ozp_a = dalloc<__nv_bfloat16>(std::max(1LL, ns), mem);
  B.ozp_erow = dalloc<int>(std::max(1LL, ne), mem);
  B.ozp_u = dalloc<__nv_bfloat16>(std::max(1LL, nu), mem);
  B.ozp_fu = dalloc<int>((long long)nsub * BMAX, mem);
  B.ozp_uoff = upload(uo, mem, D.st);
  B.ozp_nchu = nchu;
  auto slice = [&](const vector<OzMat>& mats, const float* pool, int rows, int blocks) {
    if (mats.empty() || blocks == 0) return;
    const OzMat* dm = upload(mats, mem, D.st);
    kb_oz_row_exp_a<<<dim3((rows + 7) / 8, (unsigned)mats.size()), 256, 0, D.st>>>(dm, pool, B.ozp_erow);
    CKL();
    kb_oz_slice_a<<<dim3(blocks, (unsigned)mats.size()), 256, 0, D.st>>>(dm, pool, B.ozp_erow, B.ozp_a);
    CKL();
  };
  slice(mpc, static_cast<const float*>(D.poolPC), rows_pc, blk_pc);
  slice(mpt, static_cast<const float*>(B.phit), rows_pt, blk_pt);
  vector<OzJob> jz, ju;
  for (int t = 0; t < nsub; ++t) {
    const DevSub& d = D.hs[t];
    const int nc = coarse ? d.nc : 0, n1 = nchk(d.ni);
    for (int rt = 0; rt < ntile(d.ni); ++rt) {
      const int m = std::min(OZ_M, d.ni - rt * OZ_M);
      jz.push_back(OzJob{sz[t] + rt * n1 * blk, ez[t] + rt * OZ_M, xo[t], (long long)d.rep + rt * OZ_M, t * BMAX, m,
                         n1, 0});
      if (nc > 0)
        ju.push_back(OzJob{sphi[t] + rt * nchk(nc) * blk, ephi[t] + rt * OZ_M, uo[t], (long long)d.rep + rt * OZ_M,
                           t * BMAX, m, nchk(nc), 1});
    }
  }
  // Phi^T products split along K (parts write separate planes of tc_rcs)
  auto make_jp = [&](int ks) {
    vector<OzJob> jp;
    for (int t = 0; t < nsub; ++t) {
      const DevSub& d = D.hs[t];
      const int nc = coarse ? d.nc : 0, n1 = nchk(d.ni);
      if (nc > 0 && d.ni > 0)
        for (int rt = 0; rt < ntile(nc); ++rt)
          for (int h = 0; h < ks; ++h) {  // part h: chunks [c0, c1) into plane h
            const int c0 = (int)((long long)n1 * h / ks), c1 = (int)((long long)n1 * (h + 1) / ks);
            if (c1 > c0)
              jp.push_back(OzJob{spt[t] + ((long long)rt * n1 + c0) * blk, ept[t] + rt * OZ_M, xo[t] + c0 * OZ_BB,
                                 h * ncon + d.coff + rt * OZ_M, t * BMAX, std::min(OZ_M, nc - rt * OZ_M), c1 - c0,
                                 0});
          }
    }
    return jp;
  };
  B.ozp_jz = jz.empty() ? nullptr : upload(jz, mem, D.st);
  B.ozp_ju = ju.empty() ? nullptr : upload(ju, mem, D.st);
  B.ozp_njz = (int)jz.size();
  B.ozp_nju = (int)ju.size();
  B.tc_pstride = std::max(1LL, ncon) * B.nk;
  B.tc_rcs = dalloc<double>(8 * B.tc_pstride, mem);  // room for the largest K split
  int ks = 1;
  if (!make_jp(1).empty()) {  // K split of the Phi^T product, timed on this batch's shapes
    int minch = 1 << 30;
    for (auto& d : D.hs)
      if (coarse && d.nc > 0 && d.ni > 0) minch = std::min(minch, nchk(d.ni));
    vector<int> cands = ksplit_candidates(minch);
    vector<OzJob*> lists(9, nullptr);
    vector<int> counts(9, 0);
    for (int c : cands) {
      vector<OzJob> v = make_jp(c);
      lists[c] = upload(v, mem, D.st);
      counts[c] = (int)v.size();
    }
    const std::string key = "phit_oz:" + std::to_string(nsub) + ":" + std::to_string(D.maxNI) + ":" +
                            std::to_string(D.ncpmax) + ":" + std::to_string(B.nk);
    raise_smem(kb_gemm_oz, OZ_SMEM);
    ks = tune_pick(D, key, cands, [&](int c) {
      kb_gemm_oz<<<counts[c], OZ_THREADS, OZ_SMEM, D.st>>>(lists[c], B.ozp_a, B.ozp_erow, B.oz_x, B.oz_fcol,
                                                           B.tc_rcs, B.nk, D.err, nullptr);
      CKL();
    });
    B.ozp_jp = lists[ks];
    B.ozp_njp = counts[ks];
  }
  B.tc_ks = ks;
  // planes that no job writes stay zero (the timing runs wrote into all of them)
  CK(cudaMemsetAsync(B.tc_rcs, 0, (size_t)8 * B.tc_pstride * sizeof(double), D.st));
  B.ozpc = true;
}

// out rows of every job (+)= the sliced A tile x the X chunks (kb_gemm_oz)
static void gemm_oz(Device& D, const OzJob* jobs, int njobs, const __nv_bfloat16* x, const int* fcol, double* out) {
  if (njobs <= 0) return;
  raise_smem(kb_gemm_oz, OZ_SMEM);
  kb_gemm_oz<<<njobs, OZ_THREADS, OZ_SMEM, D.st>>>(jobs, D.bt.ozp_a, D.bt.ozp_erow, x, fcol, out, D.bt.nk, D.err,
                                                   D.bt.ndone);
  CKL();
}

// out rows of every job = A tile rows x the B chunks (kb_gemm_tc3)
static void gemm_tc(Device& D, const TcJob* jobs, int njobs, const float* At, double* out, int nk,
                    const int* ndone) {
  if (njobs <= 0) return;
  raise_smem(kb_gemm_tc3, GC_SMEM);
  kb_gemm_tc3<<<std::min(njobs, D.bt.tc_grid), GC_THREADS, GC_SMEM, D.st>>>(jobs, njobs, At, D.bt.tc_b, out, nk, nk,
                                                                            D.err, ndone);
  CKL();
}

// out = addend + A B with A as hi / lo float planes (oA, oA2) and B split float2 (kb_gemm_df)
static void gemm_df(Device& D, const GemmDesc* gd, int ndesc, int maxm, const float* Ap, const float2* B, double* out,
                    const double* addend, int ldo, int nk, const int* ndone) {
  kb_gemm_df<true><<<dim3((maxm + GM - 1) / GM, ndesc), 256, 0, D.st>>>(gd, Ap, B, nk, out, addend, ldo, nk, ndone);
  CKL();
}

// The level-2 operators as hi / lo planes for the double-float products, and
// their descriptors (oA2 = the lo plane; [Z | Phi] as two single-segment products)
static void batch_prepare_l2df(Device& D, const vector<GemmDesc>& ga, const vector<GemmDesc>& gz,
                               const vector<GemmDesc>& gp, const vector<GemmDesc>& gx, long long npt, long long nuo) {
  BatchBufs& B = D.bt;
  auto& mem = B.mem;
  auto extent = [](const vector<GemmDesc>& v, bool seg2) {
    long long e = 0;
    for (auto& d : v) {
      if (d.m > 0 && d.k1 > 0) e = std::max(e, d.oA + (long long)(d.m - 1) * d.lda + d.k1);
      if (seg2 && d.m > 0 && d.k2 > 0) e = std::max(e, d.oA2 + (long long)(d.m - 1) * d.lda2 + d.k2);
    }
    return e;
  };
  auto planes = [&](const double* src, long long n) {
    float* p = dalloc<float>(2 * std::max(1LL, n), mem);
    if (n > 0) {
      kb_to_planes<<<blocks_for(n), 256, 0, D.st>>>(n, src, p);
      CKL();
    }
    return p;
  };
  auto with_lo = [](vector<GemmDesc> v, long long e) {
    for (auto& d : v) { d.oA2 = d.oA + e; d.k2 = 0; }
    return v;
  };
  const long long ea = extent(ga, false), ez = extent(gz, true), et = extent(gx, false);
  B.df_ainv = planes(D.l2_ainv, ea);
  B.df_pc = planes(static_cast<const double*>(D.poolPC), ez);
  B.df_phit = planes(static_cast<const double*>(B.phit), npt);
  B.df_t = planes(static_cast<const double*>(D.poolT), et);
  B.dA = upload(with_lo(ga, ea), mem, D.st);
  B.dP = upload(with_lo(gp, npt), mem, D.st);
  B.dX = upload(with_lo(gx, et), mem, D.st);
  B.dZ1 = upload(with_lo(gz, ez), mem, D.st);
  vector<GemmDesc> z2(gz.size());
  for (size_t t = 0; t < gz.size(); ++t) {
    const GemmDesc& d = gz[t];
    z2[t] = GemmDesc{d.oA2, d.oA2 + ez, d.ob2, 0, d.oo, d.m, d.k2, 0, d.lda2, 0, 0};
  }
  B.dZ2 = upload(z2, mem, D.st);
  B.df_fo = dalloc<float2>(std::max(1LL, nuo) * B.nk, mem);
  B.l2df = true;
}

template <typename T>
static void batch_prepare(Device& D, int nk, int lg, int maxit, int* shared_ndone, bool level2, int op = 0,
                          bool l2df = false) {
  BatchBufs& B = D.bt;
  const int ldh = std::max(maxit + 2, 2);
  // mixed level 1: op 1 slices the Schur operator (bf16 tensor cores) and runs the
  // preconditioner products as 3xTF32, op 2 slices both, op 0 runs both on the
  // SIMT pipes; op -1 takes 2 for stiff interiors (those that needed the
  // multi-step refinement), where rounding noise in the preconditioner costs
  // outer iterations, and 1 otherwise
  if (op < 0) op = D.refine_onepass ? 1 : 2;
  bool want_oz = false;
  if (D.mixed && !level2 && op >= 1) {
    want_oz = true;
    for (auto& d : D.hs) want_oz = want_oz && d.ni <= OZ_KMAX;
  }
  const bool want_ozpc = want_oz && op == 2;
  if (B.nk == nk && B.ldh >= ldh && (shared_ndone == nullptr || B.ndone == shared_ndone) && B.oz == want_oz &&
      B.ozpc == want_ozpc && B.l2df == (level2 && l2df))
    return;
  D.release_batch();
  auto& mem = B.mem;
  const long long n = D.n, nrep = D.nrep;
  long long ncon = 0, nuo = 0, nbb = 0;
  for (int t = 0; t < D.nsub; ++t) {
    ncon = std::max(ncon, (long long)D.hs[t].coff + D.hs[t].nc);
    nuo += D.hs[t].no;
    nbb += D.hs[t].NO;
  }
  const long long nc = std::max(1, D.ndofc), ldc = std::max(1, D.ldc);
  B.nk = nk;
  B.lg = lg;
  B.ldh = ldh;
  B.x = dalloc<double>(n * nk, mem);
  B.r = dalloc<double>(n * nk, mem);
  B.p = dalloc<double>(n * nk, mem);
  B.ap = dalloc<double>(n * nk, mem);
  B.z = dalloc<double>(n * nk, mem);
  B.yrep = dalloc<double>(nrep * nk, mem);
  B.zrep = dalloc<double>(nrep * nk, mem);
  B.grep = dalloc<double>(nrep * nk, mem);
  B.rcs = dalloc<double>(std::max(1LL, ncon) * nk, mem);
  B.rc = dalloc<double>(nc * nk, mem);
  B.uc = dalloc<double>(nc * nk, mem);
  B.cres = dalloc<double>(nc * nk, mem);
  B.vo = dalloc<double>(std::max(1LL, nuo) * nk, mem);
  B.part0 = dalloc<double>((long long)D.npart * nk, mem);
  B.part1 = dalloc<double>((long long)D.npart * nk, mem);
  B.part2 = dalloc<double>((long long)D.npart * nk, mem);
  B.aux = dalloc<T>(nrep * nk, mem);
  B.xs = dalloc<double>(nrep * nk, mem);  // float2 pairs or doubles: 8 bytes an entry either way
  B.ucs = dalloc<T>(std::max(1LL, ncon) * nk, mem);
  B.cbt = dalloc<double>(ldc * nk, mem);  // in the coarse inverse's precision (FP64 at most)
  B.ctl = dalloc<PcgCtl>(nk, mem);
  B.ndone = shared_ndone ? shared_ndone : dalloc<int>(1, mem);
  B.hist = dalloc<double>((long long)ldh * nk, mem);
  B.diag = dalloc<double>((long long)ldh * nk, mem);
  B.subdiag = dalloc<double>((long long)ldh * nk, mem);
  if (level2) {
    B.fo = dalloc<double>(std::max(1LL, nuo) * nk, mem);
    B.fi = dalloc<double>(nrep * nk, mem);
    B.g = dalloc<double>(n * nk, mem);
    B.bb = dalloc<double>(std::max(1LL, nbb) * BMAX, mem);
    vector<long long> ro(D.nsub);
    long long o = 0;
    for (int t = 0; t < D.nsub; ++t) {
      ro[t] = o;
      o += D.hs[t].NO;
    }
    B.rowoff = upload(ro, mem, D.st);
  }
  // GEMM descriptors: Schur operator, [Z | Phi] with the coarse solution, interior resolve, coarse inverse
  vector<GemmDesc> gs(D.nsub), gz(D.nsub), gx(D.nsub);
  vector<long long> ro(D.nsub, 0);
  {
    long long o = 0;
    for (int t = 0; t < D.nsub; ++t) { ro[t] = o; o += D.hs[t].NO; }
  }
  for (int t = 0; t < D.nsub; ++t) {
    const DevSub& d = D.hs[t];
    gs[t] = GemmDesc{d.oS, 0, d.rep, 0, d.rep, d.ni, d.ni, 0, d.NI, 0, 0};
    gz[t] = GemmDesc{d.oZ, d.oPhi, d.rep, d.coff, d.rep, d.ni, d.ni, D.ndofc > 0 ? d.nc : 0, d.NI, d.ncp, 0};
    gx[t] = GemmDesc{d.oXc, d.oXc + (long long)d.NO * d.NR, d.rep, 0, level2 ? ro[t] : D.huo_off[t],
                     d.no, d.ni, 0, d.NR, 0, 0};
  }
  vector<GemmDesc> gc(1, GemmDesc{0, 0, 0, 0, 0, D.ndofc, D.ndofc, 0, D.ldc, 0, 0});
  // Phi^T per subdomain for the coarse-residual product
  vector<GemmDesc> gp(D.nsub);
  vector<long long> opt(D.nsub);
  long long npt = 0;
  for (int t = 0; t < D.nsub; ++t) {
    const DevSub& d = D.hs[t];
    opt[t] = npt;
    gp[t] = GemmDesc{npt, 0, d.rep, 0, d.coff, d.nc, d.ni, 0, d.NI, 0, 0};
    npt += (long long)d.ncp * d.NI;
  }
  B.phit = dalloc<T>(std::max(1LL, npt), mem);
  B.gP = upload(gp, mem, D.st);
  const long long* dopt = upload(opt, mem, D.st);
  kb_phi_transpose<T><<<dim3(blocks_for((long long)D.ncpmax * D.maxNI), D.nsub), 256, 0, D.st>>>(
      D.ds, static_cast<const T*>(D.poolPC), dopt, static_cast<T*>(B.phit));
  CKL();
  B.gS = upload(gs, mem, D.st);
  B.gZ = upload(gz, mem, D.st);
  B.gX = upload(gx, mem, D.st);
  B.gC = upload(gc, mem, D.st);
  vector<GemmDesc> ga;
  if (level2 && D.l2_ainv) {  // v = A_oo^-1 f_o: the interior solves of the level-2 subdomains
    ga.resize(D.nsub);
    for (int t = 0; t < D.nsub; ++t) {
      const DevSub& d = D.hs[t];
      ga[t] = GemmDesc{D.l2_aoff[t], 0, D.huo_off[t], 0, ro[t], d.no, d.no, 0, d.NO, 0, 0};
    }
    B.gA = upload(ga, mem, D.st);
    if (l2df) batch_prepare_l2df(D, ga, gz, gp, gx, npt, nuo);
  }
  if (want_oz) {
    batch_prepare_oz(D);
    if constexpr (std::is_same_v<T, float>) {
      if (want_ozpc) batch_prepare_ozpc(D, opt);
      else batch_prepare_tc(D);
    }
  }
  if (!level2) {  // multi-column interior solves of the loads and of the interior resolve
    const int vld = D.mixed ? TC_M : NB;
    const int ncomp = D.mixed ? 3 : 1;
    vector<long long> vo(D.nsub);
    long long nv = 0;
    for (int t = 0; t < D.nsub; ++t) { vo[t] = nv; nv += (long long)ncomp * D.hs[t].NO * vld; }
    B.vb = D.mixed ? (void*)dalloc<float>(std::max(1LL, nv), mem) : (void*)dalloc<double>(std::max(1LL, nv), mem);
    B.voff = upload(vo, mem, D.st);
    B.fin = dalloc<double>(std::max(1LL, nuo) * nk, mem);
    B.ibuf = dalloc<double>(nrep * nk, mem);
    if (D.mixed) {
      vector<TcDesc> t0(D.nsub), t1(D.nsub), t2(D.nsub);
      for (int t = 0; t < D.nsub; ++t) {
        const long long comp = (long long)D.hs[t].NO * vld;
        TcDesc c = D.htd_oo[t];
        c.ncol = vld;
        c.pad = 0;
        c.oAcc = -1;
        t0[t] = c; t0[t].oB = vo[t];
        t1[t] = c; t1[t].oB = vo[t] + comp;
        t2[t] = c; t2[t].oB = vo[t] + 2 * comp; t2[t].oAcc = vo[t] + comp;  // D2 is added into D1
      }
      B.tdv0 = upload(t0, mem, D.st);
      B.tdv1 = upload(t1, mem, D.st);
      B.tdv2 = upload(t2, mem, D.st);
    } else {
      vector<BandDesc> bv(D.nsub);
      for (int t = 0; t < D.nsub; ++t) {
        bv[t] = D.hbd_oo[t];
        bv[t].ncol = vld;
        bv[t].oB = vo[t];
      }
      B.bdv = upload(bv, mem, D.st);
    }
  }
}

// vout = sum_s R_s^T S_s R_s vin for every column; partial (dotvec, vout)_w into part
template <typename T>
static void batch_schur(Device& D, const double* vin, double* vout, bool zero_fixed, const double* dotvec,
                        double* part) {
  BatchBufs& B = D.bt;
  cudaStream_t st = D.st;
  const long long cnt = (long long)D.nrep << B.lg;
  const dim3 grid((D.maxNI + GM - 1) / GM, D.nsub);
  D.prof.begin(PH_SCHUR_APPLY, st);
  if (B.oz) {
    kb_oz_col_exp<<<D.nsub, 256, 0, st>>>(D.ds, B.lg, 0, D.uniq, nullptr, vin, B.oz_fcol, B.ndone);
    CKL();
    kb_oz_slice_x<<<dim3(B.oz_nch, D.nsub), 256, 0, st>>>(D.ds, B.lg, 0, D.uniq, nullptr, vin, B.oz_fcol, B.oz_xoff,
                                                          B.oz_x, B.ndone);
    CKL();
    raise_smem(kb_schur_oz, OZ_SMEM);
    kb_schur_oz<<<dim3(B.oz_nrt, D.nsub), OZ_THREADS, OZ_SMEM, st>>>(D.ds, B.oz_s, B.oz_soff, B.oz_eoff, B.oz_erow,
                                                                    B.oz_x, B.oz_xoff, B.oz_fcol, B.yrep, B.nk, D.err,
                                                                    B.ndone);
    CKL();
  } else if (D.mixed) {
    kb_gather_df<<<blocks_for(cnt), 256, 0, st>>>(D.nrep, B.lg, D.uniq, 1.0, vin, static_cast<float2*>(B.xs), B.ndone);
    CKL();
    kb_gemm_df<false><<<grid, 256, 0, st>>>(B.gS, static_cast<const float*>(D.poolS),
                                            static_cast<const float2*>(B.xs), B.nk, B.yrep, nullptr, B.nk, B.nk,
                                            B.ndone);
    CKL();
  } else {
    kb_gather_t<double><<<blocks_for(cnt), 256, 0, st>>>(D.nrep, B.lg, D.uniq, nullptr, 1.0, vin,
                                                         static_cast<double*>(B.xs), B.ndone);
    CKL();
    gemm_t<double>(D, B.gS, D.nsub, D.maxNI, static_cast<const double*>(D.poolS), static_cast<const double*>(B.xs),
                   nullptr, B.nk, B.yrep, nullptr, B.nk, B.nk, B.ndone);
  }
  D.prof.end(PH_SCHUR_APPLY, st);
  kb_assemble_dot<<<D.npart, RT, 0, st>>>(D.n, B.lg, D.own, B.yrep, D.fixed, D.wsum, dotvec, vout, part, D.npart,
                                          zero_fixed ? 1 : 0, B.ndone);
  CKL();
}

static void batch_level2(Device& D1, const double* rc, double* uc);

// zout = BDDC preconditioner applied to every column of rin; partial (rin, zout)_w into part
template <typename T>
static void batch_pc(Device& D, const double* rin, double* zout, double* part) {
  BatchBufs& B = D.bt;
  cudaStream_t st = D.st;
  const int nk = B.nk, lg = B.lg;
  const T* pc = static_cast<const T*>(D.poolPC);
  T* aux = static_cast<T*>(B.aux);
  T* ucs = static_cast<T*>(B.ucs);
  // with the sliced Schur operator the FP32 products run on the tensor cores
  // (3xTF32) from pre-tiled A and the split B chunks, else on the FP32 SIMT pipes
  const bool tc = std::is_same_v<T, float> && B.tc_az != nullptr;
  // or with sliced blocks: FP64-exact products on the bf16 tensor cores
  const bool ozpc = std::is_same_v<T, float> && B.ozpc;
  // the level-2 device of a mixed level 1 runs its products as double-float
  const bool df = std::is_same_v<T, double> && B.l2df;
  float2* auxf = static_cast<float2*>(B.aux);
  float2* ucf = static_cast<float2*>(B.ucs);
  D.prof.begin(PH_PC_LOCAL, st);
  if (ozpc) {
    kb_oz_col_exp<<<D.nsub, 256, 0, st>>>(D.ds, lg, 0, D.uniq, D.wrep, rin, B.oz_fcol, B.ndone);
    CKL();
    kb_oz_slice_x<<<dim3(B.oz_nch, D.nsub), 256, 0, st>>>(D.ds, lg, 0, D.uniq, D.wrep, rin, B.oz_fcol, B.oz_xoff,
                                                          B.oz_x, B.ndone);
  } else if (tc) {
    kb_tile_b<<<dim3(B.tc_mch1, D.nsub), 256, 0, st>>>(1, D.ds, B.tc_boff, lg, D.uniq, D.wrep, rin, B.tc_b,
                                                        B.ndone);
  } else if (df) {
    kb_gather_df<<<blocks_for((long long)D.nrep << lg), 256, 0, st>>>(D.nrep, lg, D.uniq, 1.0, rin, auxf, B.ndone,
                                                                      D.wrep);
  } else {
    kb_gather_t<T><<<blocks_for((long long)D.nrep << lg), 256, 0, st>>>(D.nrep, lg, D.uniq, D.wrep, 1.0, rin, aux,
                                                                        B.ndone);
  }
  CKL();
  if (D.ndofc > 0) {
    if (ozpc)
      gemm_oz(D, B.ozp_jp, B.ozp_njp, B.oz_x, B.oz_fcol, B.tc_rcs);
    else if (tc)
      gemm_tc(D, B.tc_jp, B.tc_njp, B.tc_ap, B.tc_rcs, nk, B.ndone);
    else if (df)
      gemm_df(D, B.dP, D.nsub, D.ncpmax, B.df_phit, auxf, B.rcs, nullptr, nk, nk, B.ndone);
    else
      gemm_t<T>(D, B.gP, D.nsub, D.ncpmax, static_cast<const T*>(B.phit), aux, nullptr, nk, B.rcs, nullptr, nk, nk,
                B.ndone);
    kb_coarse_gather<<<blocks_for((long long)D.ndofc << lg), 256, 0, st>>>(D.ndofc, lg, D.co_ptr, D.co_sub,
                                                                           D.co_loc, D.ds,
                                                                           tc || ozpc ? B.tc_rcs : B.rcs, B.rc,
                                                                           B.ndone, tc || ozpc ? B.tc_ks : 1,
                                                                           tc || ozpc ? B.tc_pstride : 0);
    CKL();
    if (D.lev2) {
      batch_level2(D, B.rc, B.uc);
    } else {
      // explicit coarse inverse with two FP64 refinement steps, as in the single-column path
      auto coarse = [&](auto tag) {
        using TC = decltype(tag);
        const TC* minv = static_cast<const TC*>(D.cinv);
        TC* cb = static_cast<TC*>(B.cbt);
        const long long cc = (long long)D.ndofc << lg;
        kb_to_t<TC><<<blocks_for(cc), 256, 0, st>>>(cc, B.rc, cb, nk, B.ndone);
        CKL();
        gemm_t<TC>(D, B.gC, 1, D.ndofc, minv, cb, nullptr, nk, B.uc, nullptr, nk, nk, B.ndone);
        for (int rr = 0; rr < 2; ++rr) {
          kb_coarse_res<<<blocks_for(cc), 256, 0, st>>>(D.ndofc, lg, D.ac_ptr, D.ac_col, D.ac_val, B.rc, B.uc,
                                                        B.cres, B.ndone);
          CKL();
          kb_to_t<TC><<<blocks_for(cc), 256, 0, st>>>(cc, B.cres, cb, nk, B.ndone);
          CKL();
          gemm_t<TC>(D, B.gC, 1, D.ndofc, minv, cb, nullptr, nk, B.uc, B.uc, nk, nk, B.ndone);
        }
      };
      if (D.coarse64) coarse(double{});
      else coarse(T{});
    }
    if (ozpc) {
      if (B.ozp_nchu > 0) {
        kb_oz_col_exp<<<D.nsub, 256, 0, st>>>(D.ds, lg, 1, D.cmap, nullptr, B.uc, B.ozp_fu, B.ndone);
        CKL();
        kb_oz_slice_x<<<dim3(B.ozp_nchu, D.nsub), 256, 0, st>>>(D.ds, lg, 1, D.cmap, nullptr, B.uc, B.ozp_fu,
                                                                B.ozp_uoff, B.ozp_u, B.ndone);
        CKL();
      }
    } else if (tc) {
      if (B.tc_mch2 > 0) {
        kb_tile_b<<<dim3(B.tc_mch2, D.nsub), 256, 0, st>>>(2, D.ds, B.tc_boff, lg, D.cmap, nullptr, B.uc, B.tc_b,
                                                            B.ndone);
        CKL();
      }
    } else {
      long long ncon = 0;
      for (auto& d : D.hs) ncon = std::max(ncon, (long long)d.coff + d.nc);
      if (df)
        kb_gather_df<<<blocks_for(ncon << lg), 256, 0, st>>>(ncon, lg, D.cmap, 1.0, B.uc, ucf, B.ndone);
      else
        kb_gather_uc<T><<<blocks_for(ncon << lg), 256, 0, st>>>(ncon, lg, D.cmap, B.uc, ucs, B.ndone);
      CKL();
    }
  }
  // zrep = Z_s W_s r_s + Phi_s uc_s in one product per subdomain
  if (ozpc) {
    gemm_oz(D, B.ozp_jz, B.ozp_njz, B.oz_x, B.oz_fcol, B.zrep);
    gemm_oz(D, B.ozp_ju, B.ozp_nju, B.ozp_u, B.ozp_fu, B.zrep);
  } else if (tc) {
    gemm_tc(D, B.tc_jz, B.tc_njz, B.tc_az, B.zrep, nk, B.ndone);
  } else if (df) {
    gemm_df(D, B.dZ1, D.nsub, D.maxNI, B.df_pc, auxf, B.zrep, nullptr, nk, nk, B.ndone);
    if (D.ndofc > 0) gemm_df(D, B.dZ2, D.nsub, D.maxNI, B.df_pc, ucf, B.zrep, B.zrep, nk, nk, B.ndone);
  } else {
    gemm_t<T>(D, B.gZ, D.nsub, D.maxNI, pc, aux, ucs, nk, B.zrep, nullptr, nk, nk, B.ndone);
  }
  D.prof.end(PH_PC_LOCAL, st);
  kb_assemble_z<<<D.npart, RT, 0, st>>>(D.n, lg, D.own, B.zrep, D.wrep, D.wsum, rin, zout, part, D.npart, B.ndone);
  CKL();
}

// The level-1 coarse correction by one level-2 BDDC application per column
// (the batched form of level2_apply): interior solves of the level-2
// subdomains as a multi-column band solve, reduced rhs, level-2
// preconditioner with the exact level-3 coarse solve, interior resolve.
static void batch_level2(Device& D1, const double* rc, double* uc) {
  Device& D2 = *D1.lev2->dev;
  BatchBufs& B = D2.bt;
  cudaStream_t st = D1.st;
  const int nk = B.nk, lg = B.lg;
  kb_l2_fo<<<blocks_for((long long)D2.l2_nfo << lg), 256, 0, st>>>(D2.l2_nfo, lg, D2.l2_mo, rc, B.fo, B.ndone);
  CKL();
  kb_l2_fi<<<blocks_for((long long)D2.nrep << lg), 256, 0, st>>>(D2.nrep, lg, D2.l2_mi, D2.l2_wi, rc, B.fi, B.ndone);
  CKL();
  // interior solves by the explicit inverses (one product per level-2 subdomain)
  if (B.l2df) {
    long long nuo = 0;
    for (auto& d : D2.hs) nuo += d.no;
    kb_to_df<<<blocks_for(nuo << lg), 256, 0, st>>>(nuo << lg, B.fo, B.df_fo, B.ndone, nk);
    CKL();
    gemm_df(D2, B.dA, D2.nsub, D2.maxNO, B.df_ainv, B.df_fo, B.bb, nullptr, BMAX, nk, B.ndone);
  } else {
    gemm_t<double>(D2, B.gA, D2.nsub, D2.maxNO, D2.l2_ainv, B.fo, nullptr, nk, B.bb, nullptr, BMAX, nk, B.ndone);
  }
  kb_reduced_rhs<<<dim3(blocks_for((long long)D2.maxNI << lg), D2.nsub), 256, 0, st>>>(D2.ds, D2.kio, lg, B.rowoff,
                                                                                       B.bb, B.fi, B.grep, B.ndone);
  CKL();
  kb_assemble_dot<<<D2.npart, RT, 0, st>>>(D2.n, lg, D2.own, B.grep, nullptr, nullptr, nullptr, B.g, nullptr,
                                           D2.npart, 0, B.ndone);
  CKL();
  batch_pc<double>(D2, B.g, B.z, nullptr);
  // interior resolve u_o = v - X z, in place in the band block
  if (B.l2df) {
    kb_gather_df<<<blocks_for((long long)D2.nrep << lg), 256, 0, st>>>(D2.nrep, lg, D2.uniq, -1.0, B.z,
                                                                       static_cast<float2*>(B.xs), B.ndone);
    CKL();
    gemm_df(D2, B.dX, D2.nsub, D2.maxNO, B.df_t, static_cast<const float2*>(B.xs), B.bb, B.bb, BMAX, nk, B.ndone);
  } else {
    kb_gather_t<double><<<blocks_for((long long)D2.nrep << lg), 256, 0, st>>>(D2.nrep, lg, D2.uniq, nullptr, -1.0,
                                                                              B.z, static_cast<double*>(B.xs),
                                                                              B.ndone);
    CKL();
    gemm_t<double>(D2, B.gX, D2.nsub, D2.maxNO, static_cast<const double*>(D2.poolT),
                   static_cast<const double*>(B.xs), nullptr, nk, B.bb, B.bb, BMAX, nk, B.ndone);
  }
  kb_l2_out_o<<<dim3(blocks_for((long long)D2.maxNO << lg), D2.nsub), 256, 0, st>>>(D2.ds, lg, B.rowoff, D2.uo_off,
                                                                                   D2.l2_mo, B.bb, uc, B.ndone);
  CKL();
  kb_l2_out_i<<<blocks_for((long long)D2.n << lg), 256, 0, st>>>(D2.n, lg, D2.l2_mz, B.z, uc, B.ndone);
  CKL();
}

// V = A_oo^-1 F for every column (F interleaved at the interior rows): the
// tensor-core sweeps with two FP64-accurate refinement steps in mixed mode
// (the scheme of the setup's interior solves), FP64 band solves in plain mode
template <typename T>
static void batch_interior_solve(Device& D, const double* rhs) {
  BatchBufs& B = D.bt;
  cudaStream_t st = D.st;
  const int vld = D.mixed ? TC_M : NB;
  kb_v_fill<T><<<dim3(blocks_for((long long)D.maxNO * vld), D.nsub), 256, 0, st>>>(D.ds, B.lg, rhs, D.uo_off, B.voff,
                                                                                  vld, static_cast<T*>(B.vb));
  CKL();
  if constexpr (std::is_same_v<T, float>) {
    float* v = static_cast<float*>(B.vb);
    run_solve_tc(D, B.tdv0, D.nsub, D.maxnbo, vld, D.ppool_oo, v, 3, 0);
    const dim3 gr((D.maxNO + 7) / 8, D.nsub);
    kb_v_residual<<<gr, vld, 0, st>>>(D.ds, D.koo, B.lg, rhs, D.uo_off, B.voff, vld, v, 0, 1);
    CKL();
    run_solve_tc(D, B.tdv1, D.nsub, D.maxnbo, vld, D.ppool_oo, v, 3, 0);
    // as many further corrections as the setup's interior solves of the same
    // matrix needed: one one-pass correction for well-conditioned interiors,
    // else 3xTF32 corrections
    for (int step = 2; step <= D.refine_steps; ++step) {
      kb_v_residual<<<gr, vld, 0, st>>>(D.ds, D.koo, B.lg, rhs, D.uo_off, B.voff, vld, v, 1, 2);
      CKL();
      run_solve_tc(D, B.tdv2, D.nsub, D.maxnbo, vld, D.ppool_oo, v, D.refine_onepass ? 1 : 3,
                   D.refine_onepass ? 1 : 2);
    }
  } else {
    run_solve<double>(D, B.bdv, D.nsub, D.maxnbo, vld, static_cast<const double*>(D.poolT), static_cast<double*>(B.vb));
  }
}

template <typename T>
static void batch_solve_impl(Solver& S, int nrhs, double tol, int maxit, int ndecrmax, vector<int>& num_iter,
                             vector<int>& reason, vector<double>& cond) {
  Device& D = *S.dev;
  cudaStream_t st = D.st;
  const double t0 = wall_time();
  int nk = 4, lg = 2;  // at least 4 columns: the GEMM operand rows move in 16-byte pieces
  while (nk < nrhs) { nk <<= 1; ++lg; }
  batch_prepare<T>(D, nk, lg, maxit, nullptr, false, S.prm.batch_operator);
  if (D.lev2) batch_prepare<double>(*D.lev2->dev, nk, lg, 0, D.bt.ndone, true, 0, D.mixed);
  BatchBufs& B = D.bt;
  {
    double bs = 0, fm = 0, fs = 0, fp = 0;
    for (auto& d : D.hs) {
      const int nrt = (d.ni + OZ_M - 1) / OZ_M, nch = (d.ni + OZ_KC - 1) / OZ_KC;
      bs += B.oz ? (double)nrt * nch * OZ_NS * OZ_AB * 2.0 : (double)d.ni * d.NI * (D.mixed ? 8.0 : 8.0);
      fm += B.oz ? 2.0 * nrt * OZ_M * (double)nch * OZ_KC * BMAX * (OZ_NS * (OZ_NS + 1) / 2) : 0.0;
      fs += 2.0 * d.ni * (double)d.ni * nk;
      fp += 2.0 * d.ni * (double)(d.ni + 2 * d.nc) * nk;
    }
    S.stats.batch_bytes_schur = bs;
    S.stats.batch_flop_schur_mma = fm;
    S.stats.batch_flop_schur = fs;
    S.stats.batch_flop_pc = fp;
    S.stats.batch_nk = nk;
  }
  const long long n = D.n, nrep = D.nrep;
  long long nfo = 0;
  for (auto& s : S.subs) nfo += s.ndofo;
  // reduced rhs of every column g_k = f_i - A_io A_oo^-1 f_o (module_dd.f90:6995-7257)
  // from one multi-column interior solve
  vector<double> hfo((size_t)std::max(1LL, nfo) * nk, 0.0), hfi((size_t)nrep * nk, 0.0);
  {
    vector<long long> fooff(D.nsub);
    long long o = 0;
    for (int t = 0; t < D.nsub; ++t) { fooff[t] = o; o += S.subs[t].ndofo; }
#pragma omp parallel for schedule(dynamic)
    for (int t = 0; t < D.nsub; ++t) {
      const Subdomain& s = S.subs[t];
      vector<double> fo, fi;
      for (int k = 0; k < nrhs; ++k) {
        host_reduced_rhs_inputs(s, s.rhs_batch.data() + (size_t)k * s.ndof, s.rhs_batch_complete, fo, fi);
        for (int r = 0; r < s.ndofo; ++r) hfo[((size_t)fooff[t] + r) * nk + k] = fo[r];
        for (int i = 0; i < s.ndofi; ++i) hfi[((size_t)D.hs[t].rep + i) * nk + k] = fi[i];
      }
    }
  }
  vector<void*> tmp;
  CK(cudaMemcpyAsync(B.fin, hfo.data(), hfo.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(B.ibuf, hfi.data(), hfi.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  g_h2d_bytes += (double)(hfo.size() + hfi.size()) * sizeof(double);
  long long launches0 = g_launches;
  D.prof.begin(PH_SOLVE_TOTAL, st, true);
  const int vld = D.mixed ? TC_M : NB;
  batch_interior_solve<T>(D, B.fin);
  kb_v_grep<T><<<dim3(blocks_for((long long)D.maxNI << lg), D.nsub), 256, 0, st>>>(
      D.ds, D.kio, lg, B.ibuf, B.voff, vld, static_cast<const T*>(B.vb), B.grep);
  CKL();
  kb_v_out<T><<<dim3(blocks_for((long long)D.maxNO << lg), D.nsub), 256, 0, st>>>(
      D.ds, lg, B.voff, vld, static_cast<const T*>(B.vb), D.uo_off, B.vo);
  CKL();
  // initial guess: the fixed values at fixed interface dofs, zero elsewhere
  bool x0_nonzero = false;
  {
    vector<double> x0(n, 0.0);
    for (auto& s : S.subs)
      for (int i = 0; i < s.ndofi; ++i) {
        const int d = s.iivsvn[i];
        if (s.bc_present && s.ifix[d] && s.fixv[d] != 0.0) {
          x0[s.uniq[i]] = s.fixv[d];
          x0_nonzero = true;
        }
      }
    double* dx0 = dalloc<double>(n, tmp);
    CK(cudaMemcpyAsync(dx0, x0.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
    g_h2d_bytes += (double)n * sizeof(double);
    kb_bcast<<<blocks_for(n << lg), 256, 0, st>>>((int)n, lg, dx0, B.x);
    CKL();
  }
  CK(cudaMemsetAsync(B.ndone, 0, sizeof(int), st));
  CK(cudaMemsetAsync(B.diag, 0, (size_t)B.ldh * nk * sizeof(double), st));
  CK(cudaMemsetAsync(B.subdiag, 0, (size_t)B.ldh * nk * sizeof(double), st));
  // r = g (zero at fixed dofs); (g, g); r -= S x0; (r, r); p = M r; (r, p)
  kb_assemble_dot<<<D.npart, RT, 0, st>>>((int)n, lg, D.own, B.grep, D.fixed, D.wsum, nullptr, B.r, nullptr, D.npart,
                                          1, nullptr);
  CKL();
  kb_dot<<<D.npart, RT, 0, st>>>((int)n, lg, B.r, B.r, D.wsum, B.part0, D.npart);
  CKL();
  if (x0_nonzero) {
    batch_schur<T>(D, B.x, B.ap, true, nullptr, nullptr);
    kb_axpy<<<blocks_for(n << lg), 256, 0, st>>>(n << lg, -1.0, B.ap, B.r);
    CKL();
  }
  kb_dot<<<D.npart, RT, 0, st>>>((int)n, lg, B.r, B.r, D.wsum, B.part1, D.npart);
  CKL();
  batch_pc<T>(D, B.r, B.p, B.part2);
  kb_init<<<nk, RT, 0, st>>>(B.ctl, B.part0, B.part1, B.part2, D.npart, tol, maxit, ndecrmax, nrhs, B.ndone);
  CKL();
  const double tl = wall_time();
  D.prof.begin(PH_PCG, st);
  const int chunk = 2;
  int launched = 0, hdone = 0, herr = 0;
  CK(cudaMemcpyAsync(&hdone, B.ndone, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(&herr, D.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  // a bounded wait that ran out in a tensor-core kernel leaves its results
  // unusable: stop at the next poll instead of iterating on them
  while (hdone < nk && !(herr & DE_TIMEOUT)) {
    for (int q = 0; q < chunk; ++q) {
      batch_schur<T>(D, B.p, B.ap, false, B.p, B.part0);
      kb_sc_alpha<<<nk, RT, 0, st>>>(B.ctl, B.part0, D.npart);
      CKL();
      kb_update_xr<<<D.npart, RT, 0, st>>>((int)n, lg, B.ctl, B.x, B.r, B.p, B.ap, D.wsum, B.part0, D.npart);
      CKL();
      kb_sc_res<<<nk, RT, 0, st>>>(B.ctl, B.part0, D.npart, B.hist, B.ldh, B.ndone);
      CKL();
      batch_pc<T>(D, B.r, B.z, B.part0);
      kb_sc_beta<<<nk, RT, 0, st>>>(B.ctl, B.part0, D.npart, B.diag, B.subdiag, B.ldh);
      CKL();
      kb_update_p<<<blocks_for(n << lg), 256, 0, st>>>((int)n, lg, B.ctl, B.p, B.z);
      CKL();
    }
    launched += chunk;
    CK(cudaMemcpyAsync(&hdone, B.ndone, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&herr, D.err, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (launched > maxit + chunk) break;
  }
  D.prof.end(PH_PCG, st);
  S.stats.t_iterations = wall_time() - tl;
  // interior values u_o = A_oo^-1 f_o - X x for every column (module_dd.f90:6811-6932),
  // X = A_oo^-1 A_oi from the setup
  D.prof.begin(PH_POST, st);
  if (D.mixed) {
    kb_gather_df<<<blocks_for(nrep << lg), 256, 0, st>>>(nrep, lg, D.uniq, -1.0, B.x, static_cast<float2*>(B.xs),
                                                         nullptr);
    CKL();
    kb_gemm_df<true><<<dim3((D.maxNO + GM - 1) / GM, D.nsub), 256, 0, st>>>(
        B.gX, static_cast<const float*>(D.poolT), static_cast<const float2*>(B.xs), nk, B.vo, B.vo, nk, nk, nullptr);
    CKL();
  } else {
    kb_gather_t<double><<<blocks_for(nrep << lg), 256, 0, st>>>(nrep, lg, D.uniq, nullptr, -1.0, B.x,
                                                                static_cast<double*>(B.xs), nullptr);
    CKL();
    gemm_t<double>(D, B.gX, D.nsub, D.maxNO, static_cast<const double*>(D.poolT), static_cast<const double*>(B.xs),
                   nullptr, nk, B.vo, B.vo, nk, nk, nullptr);
  }
  D.prof.end(PH_POST, st);
  vector<double> hx((size_t)n * nk), hvo((size_t)std::max(1LL, nfo) * nk);
  vector<PcgCtl> hc(nk);
  vector<double> hdg((size_t)B.ldh * nk), hsd((size_t)B.ldh * nk);
  CK(cudaMemcpyAsync(hx.data(), B.x, hx.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hvo.data(), B.vo, hvo.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hc.data(), B.ctl, nk * sizeof(PcgCtl), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hdg.data(), B.diag, hdg.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(hsd.data(), B.subdiag, hsd.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  g_d2h_bytes += (double)(hx.size() + hvo.size()) * sizeof(double);
  CK(cudaMemcpyAsync(&herr, D.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  D.prof.end(PH_SOLVE_TOTAL, st);
  if (herr & DE_TIMEOUT) {
    for (void* q : tmp) cudaFreeAsync(q, st);
    // reported once: the flag is cleared so that later calls start clean
    CK(cudaMemsetAsync(D.err, 0, sizeof(int), st));
    throw Error{ERR_NUMERIC, "a bounded wait of a tensor-core kernel of the batched solve ran out"};
  }
  for (void* q : tmp) cudaFreeAsync(q, st);
  const long long launches = g_launches - launches0;
  num_iter.assign(nrhs, 0);
  reason.assign(nrhs, 0);
  cond.assign(nrhs, 1.0);
  int maxiter = 0;
  for (int k = 0; k < nrhs; ++k) {
    const PcgCtl& c = hc[k];
    num_iter[k] = c.done ? c.num_iter : maxit;
    reason[k] = c.done ? c.reason : -1;
    maxiter = std::max(maxiter, num_iter[k]);
    const int nw = c.nw;
    if (nw > 1) {
      vector<double> dg(hdg.begin() + (size_t)k * B.ldh, hdg.begin() + (size_t)k * B.ldh + nw);
      vector<double> sd(hsd.begin() + (size_t)k * B.ldh, hsd.begin() + (size_t)k * B.ldh + nw - 1);
      cond[k] = lanczos_max_eig(dg, sd);
    }
  }
  for (int t = 0; t < D.nsub; ++t) {
    Subdomain& s = S.subs[t];
    s.sol_batch.assign((size_t)s.ndof * nrhs, 0.0);
    for (int k = 0; k < nrhs; ++k) {
      double* u = s.sol_batch.data() + (size_t)k * s.ndof;
      for (int q = 0; q < s.ndofo; ++q) u[s.iovsvn[s.operm[q]]] = hvo[((size_t)D.huo_off[t] + q) * nk + k];
      for (int i = 0; i < s.ndofi; ++i) u[s.iivsvn[i]] = hx[(size_t)s.uniq[i] * nk + k];
    }
  }
  D.prof.collect();
  S.stats.h2d_bytes = g_h2d_bytes;
  S.stats.d2h_bytes = g_d2h_bytes;
  S.stats.t_solve = wall_time() - t0;
  S.stats.num_iter = maxiter;
  S.stats.launches_solve = (double)launches;
}

}  // namespace bddc
