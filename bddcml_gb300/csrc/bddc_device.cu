// GPU side of the BDDC solver: data layout in HBM, setup orchestration and
// the PCG driver.  See bddc_setup_kernels.cuh and bddc_pcg_kernels.cuh for
// the kernels and their reference counterparts.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "bddc_adaptive.cuh"
#include "bddc_batch_kernels.cuh"
#include "bddc_ozaki.cuh"
#include "bddc_batch_tc.cuh"
#include "bddc_internal.hpp"
#include "bddc_pcg_kernels.cuh"
#include "bddc_tc.cuh"

namespace bddc {

#define CK(call)                                                                                \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      throw Error{ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)};                \
  } while (0)

// Every kernel launch of the library is followed by CKL(), which also counts it.
static long long g_launches = 0;

#define CKL()                                                                                   \
  do {                                                                                          \
    ++g_launches;                                                                               \
    cudaError_t e_ = cudaGetLastError();                                                        \
    if (e_ != cudaSuccess) throw Error{ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)}; \
  } while (0)

static inline int roundup(int x, int m) { return (x + m - 1) / m * m; }

// Dynamic shared memory limits are per kernel and process, and several
// solvers (the levels of a three-level setup) launch the same kernels: the
// limit only ever grows to the largest request.
template <typename K>
static void raise_smem(K* kernel, size_t bytes) {
  static std::unordered_map<const void*, size_t> done;
  static std::mutex mu;
  std::lock_guard<std::mutex> lk(mu);
  size_t& cur = done[reinterpret_cast<const void*>(kernel)];
  if (bytes <= cur) return;
  cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void*>(kernel),
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) throw Error{ERR_CUDA, std::string("shared memory attribute: ") + cudaGetErrorString(e)};
  cur = bytes;
}

// Phase timers: CUDA events recorded on the solver's stream.  The two totals
// are always recorded; the per-phase and per-kernel slots only when profiling
// is switched on (bddcml_set_profiling_c).
struct Profiler {
  bool on = false;
  struct Rec { int ph; cudaEvent_t a, b; };
  std::vector<Rec> open, done;
  std::vector<cudaEvent_t> pool;
  double ms[NPHASE] = {0};
  int cnt[NPHASE] = {0};
  cudaEvent_t get() {
    cudaEvent_t e;
    if (!pool.empty()) { e = pool.back(); pool.pop_back(); }
    else cudaEventCreate(&e);
    return e;
  }
  void begin(int ph, cudaStream_t st, bool always = false) {
    if (!on && !always) return;
    Rec r{ph, get(), nullptr};
    cudaEventRecord(r.a, st);
    open.push_back(r);
  }
  void end(int ph, cudaStream_t st) {
    for (size_t i = open.size(); i-- > 0;)
      if (open[i].ph == ph) {
        Rec r = open[i];
        open.erase(open.begin() + i);
        r.b = get();
        cudaEventRecord(r.b, st);
        done.push_back(r);
        return;
      }
  }
  void collect() {
    for (auto& r : done) {
      cudaEventSynchronize(r.b);
      float t = 0.f;
      cudaEventElapsedTime(&t, r.a, r.b);
      ms[r.ph] += t;
      cnt[r.ph] += 1;
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    done.clear();
  }
  void reset() {
    collect();
    for (int i = 0; i < NPHASE; ++i) { ms[i] = 0; cnt[i] = 0; }
  }
  ~Profiler() {
    for (auto& r : open) { cudaEventDestroy(r.a); }
    for (auto& r : done) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
    for (auto e : pool) cudaEventDestroy(e);
  }
};

// Device memory comes from one stream-ordered CUDA memory pool per device and
// process.  The pool keeps what is freed (unlimited release threshold), so a
// later setup in the same process allocates without new mappings; memory is
// handed back to the driver by bddcml_release_device_memory_c or at exit.
// Allocations and frees are ordered on the solver's stream.
static constexpr int MAX_DEVICES = 64;
static cudaMemPool_t g_pools[MAX_DEVICES] = {};
static cudaStream_t g_alloc_st = nullptr;

static cudaMemPool_t device_pool() {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) throw Error{ERR_CUDA, "device index out of range for the memory pool table"};
  if (!g_pools[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    CK(cudaMemPoolCreate(&g_pools[dev], &props));
    uint64_t keep = UINT64_MAX;
    CK(cudaMemPoolSetAttribute(g_pools[dev], cudaMemPoolAttrReleaseThreshold, &keep));
  }
  return g_pools[dev];
}

template <typename T>
static T* dalloc(size_t n, std::vector<void*>& owned) {
  T* p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p), n * sizeof(T), device_pool(), g_alloc_st);
  if (e != cudaSuccess)
    throw Error{ERR_MEMORY, "device allocation of " + std::to_string(n * sizeof(T)) + " bytes: " +
                                cudaGetErrorString(e)};
  owned.push_back(p);
  return p;
}

// host<->device traffic of the current setup + solve (reported in the stats)
static double g_h2d_bytes = 0.0, g_d2h_bytes = 0.0;

template <typename T>
static T* upload(const T* v, size_t n, std::vector<void*>& owned, cudaStream_t st) {
  T* p = dalloc<T>(n, owned);
  if (n) CK(cudaMemcpyAsync(p, v, n * sizeof(T), cudaMemcpyHostToDevice, st));
  g_h2d_bytes += (double)n * sizeof(T);
  return p;
}

template <typename T>
static T* upload(const std::vector<T>& v, std::vector<void*>& owned, cudaStream_t st) {
  T* p = dalloc<T>(v.size(), owned);
  if (!v.empty()) CK(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
  g_h2d_bytes += (double)v.size() * sizeof(T);
  return p;
}

// Device buffers of the batched solve (nk interleaved columns), allocated at
// the first batched solve and kept until the next setup or a larger batch.
struct BatchBufs {
  int nk = 0, lg = 0, ldh = 0;
  std::vector<void*> mem;
  double *x = nullptr, *r = nullptr, *p = nullptr, *ap = nullptr, *z = nullptr;
  double *yrep = nullptr, *zrep = nullptr, *grep = nullptr, *rcs = nullptr;
  double *rc = nullptr, *uc = nullptr, *cres = nullptr, *vo = nullptr;
  double *part0 = nullptr, *part1 = nullptr, *part2 = nullptr;
  void *aux = nullptr, *xs = nullptr, *ucs = nullptr, *cbt = nullptr;  // working precision / split operands
  PcgCtl* ctl = nullptr;
  int* ndone = nullptr;  // finished columns (shared with the level-2 device)
  double *hist = nullptr, *diag = nullptr, *subdiag = nullptr;
  GemmDesc *gS = nullptr, *gZ = nullptr, *gX = nullptr, *gC = nullptr, *gP = nullptr;
  void* phit = nullptr;  // Phi^T per subdomain (working precision)
  // sliced bf16 operands of the tensor-core Schur apply (mixed mode)
  bool oz = false;
  int oz_nrt = 0, oz_nch = 0;
  __nv_bfloat16 *oz_s = nullptr, *oz_x = nullptr;
  long long *oz_soff = nullptr, *oz_eoff = nullptr, *oz_xoff = nullptr;
  int *oz_erow = nullptr, *oz_fcol = nullptr;
  // 3xTF32 tensor-core preconditioner products (with the sliced Schur operator):
  // A tiles of [Z | Phi] and of Phi^T, the B chunks of one application, job lists
  float *tc_az = nullptr, *tc_ap = nullptr, *tc_b = nullptr;
  long long* tc_boff = nullptr;
  TcJob *tc_jz = nullptr, *tc_jp = nullptr;
  int tc_njz = 0, tc_njp = 0, tc_grid = 0, tc_mch1 = 0, tc_mch2 = 0;
  int tc_ks = 1;                 // K parts of the Phi^T product, each writing its own plane of tc_rcs
  long long tc_pstride = 0;      // doubles between the planes
  double* tc_rcs = nullptr;
  // or the preconditioner products with sliced blocks (bddc_ozaki.cuh): slices of
  // Z, Phi and Phi^T, their row exponents, the sliced coarse solution of one
  // application, and the job lists (Phi^T r into the tc_rcs planes, Z r, + Phi u_c)
  bool ozpc = false;
  __nv_bfloat16 *ozp_a = nullptr, *ozp_u = nullptr;
  int *ozp_erow = nullptr, *ozp_fu = nullptr;
  long long* ozp_uoff = nullptr;
  int ozp_nchu = 0;
  OzJob *ozp_jp = nullptr, *ozp_jz = nullptr, *ozp_ju = nullptr;
  int ozp_njp = 0, ozp_njz = 0, ozp_nju = 0;
  // level-2 device only: interior loads, assembled reduced rhs, interior solutions (rows of
  // BMAX columns)
  double *fo = nullptr, *fi = nullptr, *g = nullptr, *bb = nullptr;
  GemmDesc* gA = nullptr;
  // level-2 device under a mixed level 1: the products as double-float on the
  // FP32 pipes (kb_gemm_df on hi / lo planes of the FP64 operators)
  bool l2df = false;
  float *df_ainv = nullptr, *df_pc = nullptr, *df_phit = nullptr, *df_t = nullptr;
  GemmDesc *dA = nullptr, *dZ1 = nullptr, *dZ2 = nullptr, *dP = nullptr, *dX = nullptr;
  float2* df_fo = nullptr;
  // level 1: multi-column interior solves A_oo V = F (components X0, D1, D2 of
  // NO x VB_COLS per subdomain in mixed mode, one FP64 block in plain mode)
  void* vb = nullptr;
  long long* voff = nullptr;
  TcDesc *tdv0 = nullptr, *tdv1 = nullptr, *tdv2 = nullptr;
  BandDesc* bdv = nullptr;
  double *fin = nullptr, *ibuf = nullptr;  // staged loads (interior rows, interface rows) x nk
  long long* rowoff = nullptr;
};

class Device {
 public:
  cudaStream_t st = nullptr;
  std::vector<void*> owned;    // freed on destruction / re-setup
  std::vector<void*> owned_pc; // the constraint-dependent part (rebuilt after adaptive constraints)
  void* poolP = nullptr;       // factor precision: Srho factor and [Srho^-1 | Y]
  bool mixed = true;
  int nsub = 0;
  std::vector<DevSub> hs;
  DevSub* ds = nullptr;
  // pools
  void* poolT = nullptr;   // factor precision
  void* poolPC = nullptr;  // preconditioner precision
  void* poolS = nullptr;   // Schur operator (float2 pairs or double)
  double* small = nullptr;
  // CSR blocks
  CsrView koo{}, koi{}, kio{}, kii{};
  int *c_ptr = nullptr, *c_col = nullptr;
  double* c_val = nullptr;
  int* cmap = nullptr;
  int *co_ptr = nullptr, *co_sub = nullptr, *co_loc = nullptr;
  // interface numbering
  int n = 0, nrep = 0;
  int* uniq = nullptr;
  Owners own{};
  int* fixed = nullptr;
  double *wsum = nullptr, *wrep = nullptr;
  // vectors
  double *x = nullptr, *r = nullptr, *p = nullptr, *ap = nullptr, *z = nullptr, *g = nullptr;
  double *yrep = nullptr, *zrep = nullptr, *grep = nullptr, *fi = nullptr, *fo = nullptr;
  double* zw = nullptr;  // weighted subdomain corrections w (z_s + Phi_s u_c) of one application
  float2* cvdf = nullptr;  // the coarse-solve operand as double-float pairs (FP32 coarse inverse)
  long long* fo_off = nullptr;
  double *rcpart = nullptr, *rc = nullptr, *uc = nullptr, *cres = nullptr;
  void* cinv = nullptr;            // explicit coarse inverse (factor precision, or FP64 with coarse64), ldc x ldc
  bool coarse64 = false;           // the coarse factor and inverse are FP64 (FP32 factorisation broke down)
  int refine_steps = 2;            // refinement steps the interior solves of the setup took
  bool refine_onepass = true;      // ... well-conditioned interiors (one correction)
  float refine_r1 = 0.f;           // the first correction ratio max|D1| / max|X0| of those solves
  int *ac_ptr = nullptr, *ac_col = nullptr;
  double* ac_val = nullptr;        // coarse matrix, FP64 CSR
  int ndofc = 0, ldc = 0, nrb = 0, ncpmax = 0, maxNI = 0, maxNO = 0;
  double* part = nullptr;
  int npart = 0;
  PcgCtl* ctl = nullptr;
  PcgCtl* hctl = nullptr;  // pinned
  double *hist = nullptr, *diag = nullptr, *subdiag = nullptr;
  int maxit_alloc = 0;
  double* uo = nullptr;
  long long* uo_off = nullptr;
  std::vector<long long> huo_off;
  int* err = nullptr;
  double* scal = nullptr;  // scratch scalar
  BandDesc* bd_oo = nullptr;
  std::vector<BandDesc> hbd_oo;
  bool general = false;         // matrixtype 0: LU factors and the dual coarse basis
  BandDesc* bdu_oo = nullptr;   // U^T bands of the interior LU factors (general matrices)
  std::vector<BandDesc> hbdu_oo;
  std::vector<TcDesc> htd_oo;  // tensor-core sweep descriptors of the interior systems (mixed)
  float* ppool_oo = nullptr;   // their panels
  // one-vector interior solves for new loads after setup (allocated on first use)
  void* nv_v0 = nullptr;
  void* nv_v1 = nullptr;
  void* nv_r = nullptr;
  long long* nv_off = nullptr;
  // extra interface vectors of BiCGSTAB / steepest descent (allocated on first use)
  double *kv = nullptr, *ky = nullptr, *ks = nullptr, *kt = nullptr, *krs = nullptr;
  // Krylov recycling: basis V, W = S V (n x rc_cap each), its size on the device and here
  double *rcV = nullptr, *rcW = nullptr, *rc_part = nullptr, *rc_coef = nullptr;
  int* rc_nact_dev = nullptr;
  int rc_cap = 0, rc_nact = 0;
  // three levels: the level-2 problem (on level 1), and the maps of a level-2
  // device between its layouts and the level-1 coarse dofs
  bool own_stream = true;
  Solver* lev2 = nullptr;
  int *l2_mo = nullptr, *l2_mi = nullptr, *l2_mz = nullptr;
  double* l2_ainv = nullptr;       // explicit interior inverses A_oo^-1 (NO x NO per subdomain)
  std::vector<long long> l2_aoff;  // their offsets
  double* l2_wi = nullptr;
  int l2_nfo = 0;
  int maxnbo = 0, maxw = 0, maxNR = 0;
  int nref = 0;
  BatchBufs bt;
  Profiler prof;

  ~Device() {
    release();
    if (hctl) cudaFreeHost(hctl);
    if (st) {
      cudaStreamSynchronize(st);
      if (own_stream) cudaStreamDestroy(st);
    }
    if (own_stream && g_alloc_st == st) g_alloc_st = nullptr;
  }
  void release() {
    nv_v0 = nv_v1 = nv_r = nullptr;
    kv = ky = ks = kt = krs = nullptr;
    rcV = rcW = rc_part = rc_coef = nullptr;
    rc_nact_dev = nullptr;
    rc_cap = rc_nact = 0;
    lev2 = nullptr;
    l2_mo = l2_mi = l2_mz = nullptr;
    l2_ainv = nullptr;
    l2_aoff.clear();
    l2_wi = nullptr;
    nv_off = nullptr;
    htd_oo.clear();
    ppool_oo = nullptr;
    release_batch();
    release_pc();
    for (void* q : owned) cudaFreeAsync(q, st);
    owned.clear();
    maxit_alloc = 0;
  }
  void release_batch() {
    for (void* q : bt.mem) cudaFreeAsync(q, st);
    bt = BatchBufs{};
  }
  void release_pc() {
    for (void* q : owned_pc) cudaFreeAsync(q, st);
    owned_pc.clear();
  }
};

Device* device_create(Error& err) {
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    err = Error{ERR_CUDA, std::string("no CUDA device: ") + (e == cudaSuccess ? "device count 0" : cudaGetErrorString(e))};
    return nullptr;
  }
  auto* d = new Device;
  if (cudaStreamCreateWithFlags(&d->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMallocHost(&d->hctl, sizeof(PcgCtl)) != cudaSuccess) {
    err = Error{ERR_CUDA, "stream or pinned allocation failed"};
    delete d;
    return nullptr;
  }
  g_alloc_st = d->st;
  return d;
}

Device* device_create_on_stream(Device* parent, Error& err) {
  auto* d = new Device;
  d->st = parent->st;
  d->own_stream = false;
  if (cudaMallocHost(&d->hctl, sizeof(PcgCtl)) != cudaSuccess) {
    err = Error{ERR_CUDA, "pinned allocation failed"};
    d->st = nullptr;
    delete d;
    return nullptr;
  }
  return d;
}

bool device_release_memory(Error& err) {
  try {
    CK(cudaDeviceSynchronize());
    for (auto& pool : g_pools)
      if (pool) CK(cudaMemPoolTrimTo(pool, 0));
  } catch (Error& e) {
    err = e;
    return false;
  }
  return true;
}

// Spin limit of the waits of the tensor-core sweeps on the current device
// (spins <= 0: the default).  For tests of the timeout path.
bool device_set_wait_limit(long long spins, Error& err) {
  try {
    const long long v = spins > 0 ? spins : TC_SPIN_LIMIT;
    CK(cudaMemcpyToSymbol(g_tc_wait_limit, &v, sizeof(v)));
    CK(cudaDeviceSynchronize());
  } catch (Error& e) {
    err = e;
    return false;
  }
  return true;
}

void device_destroy(Device* d) { delete d; }

// ------------------------------------------------------------ band phases
template <typename T>
static void run_factor(Device& D, const BandDesc* bd, int nbatch, int maxnb, int maxw, T* pool) {
  size_t smem = (2 * NB * (NB + 1) + 2 * SM_TILE) * sizeof(T);
  raise_smem(k_chol_diag<T>, smem);
  for (int k = 0; k < maxnb; ++k) {
    k_chol_diag<T><<<nbatch, NT, smem, D.st>>>(bd, pool, k, D.err);
    CKL();
    if (maxw > 0) {
      k_chol_off<T><<<dim3(maxw, nbatch), NT, 0, D.st>>>(bd, pool, k);
      CKL();
    }
  }
}

// Left-looking block Cholesky of FP32 band systems with the block products on
// the tensor cores: per block step the update of column k (k_chol_upd_tc,
// 3xTF32 from operand tiles made when each block was finished), the diagonal
// factor and inverse, the panel below it, and the operand tiles of the new
// column.  hbd: the host copies of the band descriptors (tile offsets).
static void run_factor_tc(Device& D, const BandDesc* bd, const vector<BandDesc>& hbd, int nbatch, int maxnb, int maxw,
                          float* pool) {
  vector<long long> toff(nbatch);
  long long nt = 0;
  for (int t = 0; t < nbatch; ++t) {
    toff[t] = nt;
    nt += (long long)hbd[t].nb * (hbd[t].w + 1) * CU_TILE;
  }
  vector<void*> tmp;
  float* tiles = dalloc<float>(std::max(1LL, nt), tmp);
  float* zero = dalloc<float>(2 * CU_HALF, tmp);
  CK(cudaMemsetAsync(zero, 0, 2 * CU_HALF * sizeof(float), D.st));
  const long long* dtoff = upload(toff, tmp, D.st);
  const size_t smem = (2 * NB * (NB + 1) + 2 * SM_TILE) * sizeof(float);
  raise_smem(k_chol_rl_diag<float>, smem);
  raise_smem(k_chol_upd_tc, CU_SMEM);
  for (int k = 0; k < maxnb; ++k) {
    if (k > 0 && maxw > 0) {
      k_chol_upd_tc<<<dim3((maxw + 2) / 2, nbatch), CU_THREADS, CU_SMEM, D.st>>>(bd, pool, tiles, dtoff, zero, k,
                                                                                   D.err);
      CKL();
    }
    k_chol_rl_diag<float><<<nbatch, NT, smem, D.st>>>(bd, pool, k, D.err);
    CKL();
    const int m = std::min(maxw, maxnb - 1 - k);
    if (m > 0) {
      k_chol_rl_panel<float><<<dim3(m, nbatch), NT, 0, D.st>>>(bd, pool, k);
      CKL();
    }
    if (k < maxnb - 1) {
      k_chol_tile<<<dim3(maxw + 1, nbatch), 256, 0, D.st>>>(bd, pool, dtoff, tiles, k);
      CKL();
    }
  }
  for (void* q : tmp) cudaFreeAsync(q, D.st);
}

// right-looking block Cholesky (k_chol_rl_*): for a few dense systems
template <typename T>
static void run_factor_rl(Device& D, const BandDesc* bd, int nbatch, int maxnb, int maxw, T* pool, int* err) {
  size_t smem = (2 * NB * (NB + 1) + 2 * SM_TILE) * sizeof(T);
  raise_smem(k_chol_rl_diag<T>, smem);
  for (int k = 0; k < maxnb; ++k) {
    k_chol_rl_diag<T><<<nbatch, NT, smem, D.st>>>(bd, pool, k, err);
    CKL();
    const int m = std::min(maxw, maxnb - 1 - k);
    if (m > 0) {
      k_chol_rl_panel<T><<<dim3(m, nbatch), NT, 0, D.st>>>(bd, pool, k);
      CKL();
      k_chol_rl_update<T><<<dim3(m * (m + 1) / 2, nbatch), NT, 0, D.st>>>(bd, pool, k);
      CKL();
    }
  }
}

// block LU of general band matrices: L and U^T bands (k_lu_diag / k_lu_off)
template <typename T>
static void run_factor_lu(Device& D, const BandDesc* bl, const BandDesc* bu, int nbatch, int maxnb, int maxw,
                          T* pool) {
  size_t smem = (2 * NB * (NB + 1) + 2 * SM_TILE) * sizeof(T);
  raise_smem(k_lu_diag<T>, smem);
  for (int k = 0; k < maxnb; ++k) {
    k_lu_diag<T><<<nbatch, NT, smem, D.st>>>(bl, bu, pool, k, D.err);
    CKL();
    if (maxw > 0) {
      k_lu_off<T><<<dim3(maxw, nbatch), NT, 0, D.st>>>(bl, bu, pool, k);
      CKL();
    }
  }
}

// FP32 factors: panels for the tensor-core sweeps (after the factorisation);
// backward panels from bdb (U^T of a general matrix) when given
static void run_panels(Device& D, const BandDesc* bd, const TcDesc* td, int nbatch, int maxnb, int maxw,
                       const float* L, float* P, const BandDesc* bdb = nullptr) {
  k_make_panels<<<dim3(maxw + 1, maxnb, nbatch), NT, 0, D.st>>>(bd, td, L, P, bdb);
  CKL();
}

// forward + backward sweeps on the tensor cores (3xTF32, TMEM accumulation):
// one launch per direction, one CTA per (system, 128-column tile)
// forward + backward tensor-core sweep; passes 3 (3xTF32) or 1 (TF32); with
// acc the backward sweep also adds its result into each system's oAcc block
template <int PASSES, int ACC>
static void sweep_pair(Device& D, dim3 grid, const TcDesc* td, const float* P, float* B, int* maxabs) {
  static bool attr = false;
  const size_t smem = tc_smem_bytes();
  if (!attr) {  // both instances launched here need the large shared-memory window
    CK(cudaFuncSetAttribute(k_band_sweep_tc<PASSES, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CK(cudaFuncSetAttribute(k_band_sweep_tc<PASSES, 0>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    CK(cudaFuncSetAttribute(k_band_sweep_tc<PASSES, ACC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CK(cudaFuncSetAttribute(k_band_sweep_tc<PASSES, ACC>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    attr = true;
  }
  k_band_sweep_tc<PASSES, 0><<<grid, SW_THREADS, smem, D.st>>>(td, P, B, 0, D.err, nullptr);
  CKL();
  k_band_sweep_tc<PASSES, ACC><<<grid, SW_THREADS, smem, D.st>>>(td, P, B, 1, D.err, maxabs);
  CKL();
}

// acc: 0 none, 1 add into oAcc, 2 add into the renormalised pair ending at oAcc
// maxabs (optional, one int per system): the largest |result| of each
// system, as FP32 bits, merged into the array by atomicMax
static void run_solve_tc(Device& D, const TcDesc* td, int nbatch, int maxnb, int maxncol, const float* P, float* B,
                         int passes = 3, int acc = 0, int* maxabs = nullptr) {
  (void)maxnb;
  dim3 grid(maxncol / TC_M, nbatch);
  if (passes == 3 && acc == 2) sweep_pair<3, 2>(D, grid, td, P, B, maxabs);
  else if (passes == 3 && acc == 1) sweep_pair<3, 1>(D, grid, td, P, B, maxabs);
  else if (passes == 3) sweep_pair<3, 0>(D, grid, td, P, B, maxabs);
  else if (acc) sweep_pair<1, 1>(D, grid, td, P, B, maxabs);
  else sweep_pair<1, 0>(D, grid, td, P, B, maxabs);
}

template <typename T>
static void run_solve(Device& D, const BandDesc* bd, int nbatch, int maxnb, int maxncol, const T* L, T* B,
                      const BandDesc* bdb = nullptr) {
  dim3 grid(maxncol / NB, nbatch);
  for (int k = 0; k < maxnb; ++k) {
    k_trsm_fwd<T><<<grid, NT, 0, D.st>>>(bd, L, B, k);
    CKL();
  }
  for (int k = maxnb - 1; k >= 0; --k) {  // backward with L^T, or with U (its transposed band) when bdb is given
    k_trsm_bwd<T><<<grid, NT, 0, D.st>>>(bdb ? bdb : bd, L, B, k);
    CKL();
  }
}

// FP32 flop of one forward + backward block-band sweep over ncol columns
// MMA work of one forward + backward sweep pair of k_band_sweep_tc, counting
// the block rows each 128-column tile processes: a tile inside the pad leading
// identity columns starts its forward sweep at its diagonal block row, and with
// `lower` also ends its backward sweep there
static double band_sweep_flop(int nb, int w, int ncol, int pad = 0, bool lower = false) {
  double f = 0.0;
  for (int c0 = 0; c0 < ncol; c0 += TC_M) {
    const int s = c0 + TC_M <= pad ? c0 / NB : 0;
    for (int k = s; k < nb; ++k) f += 2.0 * NB * TC_M * NB * (std::min(k, w) + 1);
    for (int k = lower ? s : 0; k < nb; ++k) f += 2.0 * NB * TC_M * NB * (std::min(w, nb - 1 - k) + 1);
  }
  return f;
}

template <typename T>
static void setup_numeric(Solver& S, Device& D, vector<SubBlocks>& blk);
template <typename T>
static void setup_precond(Solver& S, Device& D);
template <typename T>
static void adaptive_constraints(Solver& S, Device& D);
template <typename T>
static void setup_level2(Solver& S, Device& D);
template <typename T>
static vector<vector<double>> coarse_energies(Device& D, const vector<int>& subs, vector<vector<double>>* phis);

bool device_setup(Solver& S, Error& err) {
  Device& D = *S.dev;
  try {
    S.lev2.reset();  // the previous level-2 state shares this device's stream
    D.release();
    D.prof.reset();
    g_h2d_bytes = 0.0;
    g_d2h_bytes = 0.0;
    g_launches = 0;
    D.mixed = S.prm.precision != 0;
    double t0 = wall_time();
    int nsub = (int)S.subs.size();
    D.nsub = nsub;
    vector<SubBlocks>& blk = S.blocks;
    for (int t = 0; t < nsub; ++t) {
      auto& b = blk[t];
      // the double-float residual and Schur kernels stage a row in shared memory
      if (D.mixed && (b.maxrow_oo > 96 || b.maxrow_oi > 95 || b.maxrow_io > 128 || b.maxrow_ii > 128))
        throw Error{ERR_UNSUPPORTED, "subdomain matrix rows longer than the staging buffers (96/128 entries)"};
      if (S.subs[t].ndofi == 0) throw Error{ERR_ARGUMENT, "subdomain without interface"};
    }
    S.stats.t_host_setup += wall_time() - t0;
    double t1 = wall_time();
    if (D.mixed) {
      setup_numeric<float>(S, D, blk);
      setup_precond<float>(S, D);
      if (S.prm.use_adaptive) {
        adaptive_constraints<float>(S, D);
        setup_precond<float>(S, D);
      }
      if (S.prm.nlevels == 3) setup_level2<float>(S, D);
    } else {
      setup_numeric<double>(S, D, blk);
      setup_precond<double>(S, D);
      if (S.prm.use_adaptive) {
        adaptive_constraints<double>(S, D);
        setup_precond<double>(S, D);
      }
      if (S.prm.nlevels == 3) setup_level2<double>(S, D);
    }
    vector<SubBlocks>().swap(S.blocks);
    // check device error flags
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, D.err, sizeof(int), cudaMemcpyDeviceToHost, D.st));
    CK(cudaStreamSynchronize(D.st));
    if (herr & DE_TIMEOUT) {
      CK(cudaMemsetAsync(D.err, 0, sizeof(int), D.st));
      throw Error{ERR_NUMERIC, "a bounded wait of a tensor-core kernel of the setup ran out (flags " +
                                   std::to_string(herr) + ")"};
    }
    if (herr) throw Error{ERR_NUMERIC, "non-positive pivot in a subdomain or coarse factorisation (flags " +
                                            std::to_string(herr) + ")"};
    D.prof.collect();
    S.stats.t_device_setup = wall_time() - t1;
    S.stats.launches_setup = (double)g_launches;
  } catch (Error& e) {
    err = e;
    return false;
  }
  return true;
}

template <typename T>
static void setup_numeric(Solver& S, Device& D, vector<SubBlocks>& blk) {
  const int nsub = D.nsub;
  cudaStream_t st = D.st;
  auto& own = D.owned;
  D.nref = D.mixed ? 2 : 0;
  D.general = S.prm.matrixtype == 0;

  // ---- sizes and offsets
  D.hs.assign(nsub, DevSub{});
  long long oT = 0, oS = 0, oPan = 0;
  vector<std::array<long long, 2>> poff(nsub, {0, 0});
  int rep = 0, koo = 0, koi = 0, kio = 0, kii = 0;
  D.maxnbo = 0; D.maxw = 0; D.maxNR = 0; D.maxNI = 0; D.maxNO = 0;
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    auto& b = blk[t];
    DevSub d{};
    d.no = s.ndofo; d.ni = s.ndofi;
    d.NO = roundup(d.no, NB); d.NI = roundup(d.ni, NB);
    d.NR = roundup(d.ni + 1, TC_M);
    d.nbo = d.NO / NB; d.w = b.w; d.nbi = d.NI / NB; d.nref = D.nref;
    d.oL = oT; oT += (long long)d.nbo * (d.w + 1) * NB * NB;
    d.oLinv = oT; oT += (long long)d.nbo * NB * NB;
    if (D.general) {
      d.oU = oT; oT += (long long)d.nbo * (d.w + 1) * NB * NB;
      d.oUinv = oT; oT += (long long)d.nbo * NB * NB;
    }
    d.oXc = oT; oT += (long long)(d.nref == 0 ? 1 : (d.nref == 1 ? 2 : 3)) * d.NO * d.NR;
    if (std::is_same_v<T, float>) {
      poff[t][0] = oPan; oPan += (long long)d.nbo * (d.w + 1) * 2 * TC_PCHUNK;
      poff[t][1] = oPan; oPan += (long long)d.nbo * (d.w + 1) * 2 * TC_PCHUNK;
    }
    d.oS = oS; oS += (long long)d.NI * d.NI;
    d.rep = rep; rep += d.NI;
    d.koo = koo; koo += d.no + 1;
    d.koi = koi; koi += d.no + 1;
    d.kio = kio; kio += d.ni + 1;
    d.kii = kii; kii += d.ni + 1;
    d.rho = b.rho;
    D.hs[t] = d;
    D.maxnbo = std::max(D.maxnbo, d.nbo); D.maxw = std::max(D.maxw, d.w);
    D.maxNR = std::max(D.maxNR, d.NR); D.maxNI = std::max(D.maxNI, d.NI); D.maxNO = std::max(D.maxNO, d.NO);
  }
  D.nrep = rep;
  {
    S.stats.flop_sweep_oo = S.stats.bytes_residual = S.stats.bytes_schur_apply = 0;
    for (auto& d : D.hs) {
      S.stats.flop_sweep_oo += band_sweep_flop(d.nbo, d.w, d.NR);
      S.stats.bytes_residual += (double)d.NO * d.NR * 4.0 * 3.0;
      S.stats.bytes_schur_apply += (double)d.ni * d.NI * 8.0 + d.ni * 16.0;
    }
  }
  S.stats.bytes_per_iteration = 0;
  for (auto& d : D.hs)
    S.stats.bytes_per_iteration += (double)d.NI * d.NI * (D.mixed ? (8.0 + 4.0) : 16.0);

  // ---- allocations
  double tw0 = wall_time();
  D.poolT = dalloc<T>(oT, own);
  float* ppool = std::is_same_v<T, float> ? dalloc<float>(oPan, own) : nullptr;
  D.poolS = D.mixed ? (void*)dalloc<float2>(oS, own) : (void*)dalloc<double>(oS, own);
  D.err = dalloc<int>(1, own);
  S.stats.t_dev_alloc = wall_time() - tw0;
  CK(cudaMemsetAsync(D.err, 0, sizeof(int), st));
  CK(cudaMemsetAsync(D.poolT, 0, oT * sizeof(T), st));
  D.ds = upload(D.hs, own, st);

  // ---- CSR blocks: every subdomain's rows (ptr with nrow + 1 entries,
  // shifted by the subdomain's first entry) concatenated into one staging
  // buffer, filled by all host threads (first touch included), then copied
  // in one transfer.  The per-subdomain arrays are released as they are copied.
  auto concat = [&](auto get_ptr, auto get_col, auto get_val, CsrView& view) {
    vector<long long> po(nsub + 1, 0), co(nsub + 1, 0);
    for (int t = 0; t < nsub; ++t) {
      po[t + 1] = po[t] + (long long)get_ptr(blk[t]).size();
      co[t + 1] = co[t] + (long long)get_col(blk[t]).size();
    }
    if (co[nsub] > INT32_MAX) throw Error{ERR_UNSUPPORTED, "more than 2^31 matrix entries in one block type"};
    std::unique_ptr<int[]> ptr(new int[std::max<long long>(1, po[nsub])]);
    std::unique_ptr<int[]> col(new int[std::max<long long>(1, co[nsub])]);
    std::unique_ptr<double[]> val(new double[std::max<long long>(1, co[nsub])]);
#pragma omp parallel for schedule(dynamic)
    for (int t = 0; t < nsub; ++t) {
      auto& p = get_ptr(blk[t]);
      auto& c = get_col(blk[t]);
      auto& v = get_val(blk[t]);
      const int base = (int)co[t];
      for (size_t i = 0; i < p.size(); ++i) ptr[po[t] + i] = base + p[i];
      if (!c.empty()) {
        std::memcpy(col.get() + co[t], c.data(), c.size() * sizeof(int));
        std::memcpy(val.get() + co[t], v.data(), v.size() * sizeof(double));
      }
      std::decay_t<decltype(p)>().swap(p);
      std::decay_t<decltype(c)>().swap(c);
      std::decay_t<decltype(v)>().swap(v);
    }
    view.ptr = upload(ptr.get(), (size_t)po[nsub], own, st);
    view.col = upload(col.get(), (size_t)co[nsub], own, st);
    view.val = upload(val.get(), (size_t)co[nsub], own, st);
  };
  concat([](SubBlocks& b) -> vector<int>& { return b.oo_ptr; }, [](SubBlocks& b) -> rawvec<int>& { return b.oo_col; },
         [](SubBlocks& b) -> rawvec<double>& { return b.oo_val; }, D.koo);
  concat([](SubBlocks& b) -> vector<int>& { return b.oi_ptr; }, [](SubBlocks& b) -> rawvec<int>& { return b.oi_col; },
         [](SubBlocks& b) -> rawvec<double>& { return b.oi_val; }, D.koi);
  concat([](SubBlocks& b) -> vector<int>& { return b.io_ptr; }, [](SubBlocks& b) -> rawvec<int>& { return b.io_col; },
         [](SubBlocks& b) -> rawvec<double>& { return b.io_val; }, D.kio);
  concat([](SubBlocks& b) -> vector<int>& { return b.ii_ptr; }, [](SubBlocks& b) -> rawvec<int>& { return b.ii_col; },
         [](SubBlocks& b) -> rawvec<double>& { return b.ii_val; }, D.kii);
  // ---- interface vectors and owner lists
  D.n = S.ninterface;
  {
    vector<int> uq(D.nrep, 0);
    vector<double> wr(D.nrep, 0.0), fir(D.nrep, 0.0), fov;
    vector<long long> fooff(nsub), uooff(nsub);
    long long fpos = 0;
    for (int t = 0; t < nsub; ++t) {
      auto& s = S.subs[t];
      auto& d = D.hs[t];
      for (int i = 0; i < s.ndofi; ++i) { uq[d.rep + i] = s.uniq[i]; wr[d.rep + i] = s.wi[i]; fir[d.rep + i] = blk[t].fi[i]; }
      fooff[t] = fpos;
      uooff[t] = fpos;
      fov.insert(fov.end(), blk[t].fo.begin(), blk[t].fo.end());
      fpos += s.ndofo;
    }
    D.uniq = upload(uq, own, st);
    D.wrep = upload(wr, own, st);
    D.fi = upload(fir, own, st);
    D.fo = upload(fov, own, st);
    D.fo_off = upload(fooff, own, st);
    D.uo_off = upload(uooff, own, st);
    D.huo_off = uooff;
    D.uo = dalloc<double>(fpos, own);
    vector<int> optr(D.n + 1, 0), orep, osub, oloc;
    for (int t = 0; t < nsub; ++t) for (int u : S.subs[t].uniq) optr[u + 1]++;
    for (int u = 0; u < D.n; ++u) optr[u + 1] += optr[u];
    orep.resize(optr[D.n]); osub.resize(optr[D.n]); oloc.resize(optr[D.n]);
    vector<int> pos(optr.begin(), optr.end() - 1);
    for (int t = 0; t < nsub; ++t)
      for (int i = 0; i < S.subs[t].ndofi; ++i) {
        int u = S.subs[t].uniq[i];
        orep[pos[u]] = D.hs[t].rep + i; osub[pos[u]] = t; oloc[pos[u]++] = i;
      }
    D.own.ptr = upload(optr, own, st);
    D.own.rep = upload(orep, own, st);
    D.own.sub = upload(osub, own, st);
    D.own.loc = upload(oloc, own, st);
    D.fixed = upload(S.iface_fixed, own, st);
    D.wsum = upload(S.iface_wsum, own, st);
  }
  D.x = dalloc<double>(D.n, own); D.r = dalloc<double>(D.n, own); D.p = dalloc<double>(D.n, own);
  D.ap = dalloc<double>(D.n, own); D.z = dalloc<double>(D.n, own); D.g = dalloc<double>(D.n, own);
  D.yrep = dalloc<double>(D.nrep, own); D.zrep = dalloc<double>(D.nrep, own); D.grep = dalloc<double>(D.nrep, own);
  D.zw = dalloc<double>(D.nrep, own);
  CK(cudaMemsetAsync(D.yrep, 0, D.nrep * sizeof(double), st));
  CK(cudaMemsetAsync(D.zrep, 0, D.nrep * sizeof(double), st));
  CK(cudaMemsetAsync(D.grep, 0, D.nrep * sizeof(double), st));
  D.nrb = (D.maxNI + AROWS - 1) / AROWS;
  D.npart = std::min(MAXPART, std::max(1, (D.n + RT - 1) / RT));
  D.part = dalloc<double>(MAXPART, own);
  D.ctl = dalloc<PcgCtl>(1, own);
  D.scal = dalloc<double>(4, own);

  T* poolT = static_cast<T*>(D.poolT);
  if (D.mixed)
    raise_smem(k_schur_apply_df, D.maxNI * sizeof(float2));
  else
    raise_smem(k_schur_apply_f64, D.maxNI * sizeof(double));
  raise_smem(k_pc_local<T>, D.maxNI * sizeof(typename PcVec<T>::type));
  raise_smem(k_post_df, (D.maxNI + 1) * sizeof(float2));
  (void)ppool;

  // ---- interior band factor
  D.hbd_oo.resize(nsub);
  for (int t = 0; t < nsub; ++t) {
    auto& d = D.hs[t];
    D.hbd_oo[t] = BandDesc{d.nbo, d.w, d.NR, 0, d.oL, d.oLinv, d.oXc};
  }
  D.bd_oo = upload(D.hbd_oo, own, st);
  D.hbdu_oo.clear();
  D.bdu_oo = nullptr;
  if (D.general) {
    D.hbdu_oo = D.hbd_oo;
    for (int t = 0; t < nsub; ++t) { D.hbdu_oo[t].oL = D.hs[t].oU; D.hbdu_oo[t].oLinv = D.hs[t].oUinv; }
    D.bdu_oo = upload(D.hbdu_oo, own, st);
  }
  S.stats.t_dev_h2d = wall_time() - tw0 - S.stats.t_dev_alloc;
  D.prof.begin(PH_NUMERIC_TOTAL, st, true);
  D.prof.begin(PH_FACTOR_OO, st);
  if (D.general) {
    k_fill_band_lu<T><<<dim3((D.maxNO + 127) / 128, nsub), 128, 0, st>>>(D.ds, D.koo, poolT, D.bd_oo, D.bdu_oo);
    CKL();
    run_factor_lu<T>(D, D.bd_oo, D.bdu_oo, nsub, D.maxnbo, D.maxw, poolT);
  } else {
    k_fill_band<T><<<dim3((D.maxNO + 127) / 128, nsub), 128, 0, st>>>(D.ds, D.koo, poolT, D.bd_oo);
    CKL();
    // SIMT FP32 products: the interior factor's rounding sets the first
    // refinement ratio r1 (8e-6 at 16^3), and 3xTF32 block updates raise it
    // (to 8.5e-6) together with the error left after the first correction
    // (2.3e-8 -> 6e-8 of the oracle's solution at 128^3); the band updates
    // are also too small (K <= 64 w) to gain from the tensor cores
    run_factor<T>(D, D.bd_oo, nsub, D.maxnbo, D.maxw, poolT);
  }
  vector<TcDesc> htd(nsub);
  TcDesc* td_oo = nullptr;
  if constexpr (std::is_same_v<T, float>) {
    for (int t = 0; t < nsub; ++t) {
      auto& d = D.hs[t];
      htd[t] = TcDesc{d.nbo, d.w, d.NR, 0, d.oXc, poff[t][0], poff[t][1], -1};
    }
    td_oo = upload(htd, own, st);
    run_panels(D, D.bd_oo, td_oo, nsub, D.maxnbo, D.maxw, poolT, ppool, D.bdu_oo);
    D.htd_oo = htd;
    D.ppool_oo = ppool;
  }
  D.prof.end(PH_FACTOR_OO, st);
  // ---- interior solves [X | v] = A_oo^-1 [A_oi | f_o], refined in mixed precision
  int* dmax = nullptr;  // mixed precision: per refinement step and system, max |result| as FP32 bits
  if (std::is_same_v<T, float>) {
    dmax = dalloc<int>((size_t)nsub * 8, own);
    CK(cudaMemsetAsync(dmax, 0, (size_t)nsub * 8 * sizeof(int), st));
  }
  D.prof.begin(PH_SOLVE_OO, st);
  k_fill_rhs<T><<<dim3((D.maxNO + 127) / 128, nsub), 128, 0, st>>>(D.ds, D.koi, D.fo, D.fo_off, poolT);
  CKL();
  if constexpr (std::is_same_v<T, float>) run_solve_tc(D, td_oo, nsub, D.maxnbo, D.maxNR, ppool, poolT, 3, 0, dmax);
  else run_solve<T>(D, D.bd_oo, nsub, D.maxnbo, D.maxNR, poolT, poolT, D.bdu_oo);
  D.prof.end(PH_SOLVE_OO, st);
  // Mixed precision: refinement with FP64-accurate residuals until the
  // correction is negligible (iterative refinement in the sense of Wilkinson;
  // each step contracts the error by about kappa(A_oo) eps_fp32):
  //   R0 = [A_oi | f_o] - A_oo X0 in double-float -> component 1 (and 2),
  //   D1 = A_oo^-1 R0 in place (3xTF32), r1 = max|D1| / max|X0|.
  //   If r1 <= 1e-5 (well-conditioned interiors) X0 + D1 is accurate to about
  //     r1^2 <= 1e-10 and the refinement stops.
  //   Otherwise: residuals of the pair X0 + D in double-float and 3xTF32
  //     corrections added into the pair (renormalised), until
  //     max|correction| / max|X0| <= 1e-12 (at most 13 corrections).
  // X is the FP32 pair (X0, D) in components 0 and 1.
  if constexpr (std::is_same_v<T, float>) {
    // per-subdomain max|correction| / max|X0| of slot `slot`
    auto ratios = [&](int slot) {
      vector<int> hmax((size_t)nsub * 8);
      CK(cudaMemcpyAsync(hmax.data(), dmax, hmax.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      vector<float> r(nsub, 0.f);
      for (int t = 0; t < nsub; ++t) {
        float x0, dd;
        std::memcpy(&x0, &hmax[t], 4);
        std::memcpy(&dd, &hmax[(size_t)slot * nsub + t], 4);
        if (x0 > 0) r[t] = dd / x0;
      }
      return r;
    };
    auto ratio = [&](int slot) {
      const vector<float> r = ratios(slot);
      return nsub ? *std::max_element(r.begin(), r.end()) : 0.f;
    };
    // sweep descriptors for components (comp, acc_comp); systems with act[t] == 0 are skipped
    auto tds = [&](int comp, int acc_comp, const vector<char>* act = nullptr) {
      vector<TcDesc> h2 = htd;
      for (int t = 0; t < nsub; ++t) {
        const long long cs = (long long)D.hs[t].NO * D.hs[t].NR;
        h2[t].oB = D.hs[t].oXc + comp * cs;
        h2[t].oAcc = acc_comp >= 0 ? D.hs[t].oXc + acc_comp * cs : -1;
        if (act && !(*act)[t]) h2[t].nb = 0;
      }
      return upload(h2, own, st);
    };
    const dim3 gres((D.maxNO + RES_ROWS - 1) / RES_ROWS, nsub);
    D.prof.begin(PH_RESIDUAL, st);
    k_residual_df<<<gres, 128, 0, st>>>(D.ds, D.koo, D.koi, D.fo, D.fo_off, poolT, 0, 1, 2);
    CKL();
    D.prof.end(PH_RESIDUAL, st);
    D.prof.begin(PH_SOLVE_OO, st);
    run_solve_tc(D, tds(1, -1), nsub, D.maxnbo, D.maxNR, ppool, poolT, 3, 0, dmax + nsub);
    D.prof.end(PH_SOLVE_OO, st);
    const float r1 = ratio(1);
    float rl = r1;
    int steps = 1;
    if (r1 <= 1e-5f) {
      // Well-conditioned interiors (Poisson: r1 = 8e-6 at 16^3): a 3xTF32 solve
      // is accurate to about r1 of its result, so the error left in X0 + D1 is
      // about r1^2 <= 1e-10 of X; with the amplification by the Schur
      // complement's cancellation (a few hundred at 128^3) the solution stays
      // within the 1e-7 tolerance of the mixed path; no further correction.
    } else {
      // The contraction per step is about kappa(A_oo) u with u ~ 2^-21 for the
      // 3xTF32 sweeps (two TF32 halves per operand, the lo x lo term dropped):
      // interiors with kappa ~ 1e5 (stiff inclusions) contract by ~0.2 a step.
      // A subdomain whose correction has dropped below 1e-12 of its solution
      // leaves the loop (its residual and sweeps are skipped): the stiff ones
      // take all the steps, the others two or three.
      vector<char> act(nsub, 1);
      const vector<float> rr1 = ratios(1);
      for (int t = 0; t < nsub; ++t) act[t] = rr1[t] > 1e-12f;
      vector<int> hact(nsub);
      int* dact = dalloc<int>(std::max(1, nsub), own);
      for (int step = 2; step <= 14 && rl > 1e-12f; ++step) {
        for (int t = 0; t < nsub; ++t) hact[t] = act[t];
        CK(cudaMemcpyAsync(dact, hact.data(), (size_t)nsub * sizeof(int), cudaMemcpyHostToDevice, st));
        D.prof.begin(PH_RESIDUAL, st);
        k_residual_df<<<gres, 128, 0, st>>>(D.ds, D.koo, D.koi, D.fo, D.fo_off, poolT, 1, 2, -1, dact);
        CKL();
        D.prof.end(PH_RESIDUAL, st);
        D.prof.begin(PH_SOLVE_OO, st);
        CK(cudaMemsetAsync(dmax + 2 * nsub, 0, (size_t)nsub * sizeof(int), st));
        run_solve_tc(D, tds(2, 1, &act), nsub, D.maxnbo, D.maxNR, ppool, poolT, 3, 2, dmax + 2 * nsub);
        D.prof.end(PH_SOLVE_OO, st);
        const vector<float> r = ratios(2);
        rl = 0.f;
        for (int t = 0; t < nsub; ++t)
          if (act[t]) {
            rl = std::max(rl, r[t]);
            if (r[t] <= 1e-12f) act[t] = 0;
          }
        steps = step;
      }
    }
    S.stats.refine1 = r1;
    S.stats.refine2 = rl;
    S.stats.refine_steps = steps;
    D.refine_steps = steps;
    D.refine_onepass = r1 <= 1e-5f;
    D.refine_r1 = r1;
  }
  // ---- Schur complements and the subdomain reduced rhs
  D.prof.begin(PH_SCHUR, st);
  if (D.mixed) {
    k_schur_df<<<dim3(D.maxNI, nsub), 128, 0, st>>>(D.ds, D.kio, D.kii, reinterpret_cast<const float*>(poolT),
                                                    static_cast<float2*>(D.poolS), D.fi, D.grep);
    CKL();
    if (!D.general) {
      k_symmetrize<float2><<<dim3(D.maxNI / 32, D.maxNI / 32, nsub), dim3(32, 8), 0, st>>>(
          D.ds, static_cast<float2*>(D.poolS), 0);
      CKL();
    }
  } else {
    k_schur_f64<<<dim3(D.maxNI, nsub), 128, 0, st>>>(D.ds, D.kio, D.kii, reinterpret_cast<const double*>(poolT),
                                                     static_cast<double*>(D.poolS), D.fi, D.grep);
    CKL();
    if (!D.general) {
      k_symmetrize<double><<<dim3(D.maxNI / 32, D.maxNI / 32, nsub), dim3(32, 8), 0, st>>>(
          D.ds, static_cast<double*>(D.poolS), 0);
      CKL();
    }
  }
  D.prof.end(PH_SCHUR, st);
  // ---- assembled reduced rhs (module_dd.f90:7090-7135)
  k_assemble_plain<<<(D.n + 255) / 256, 256, 0, st>>>(D.n, D.own, D.grep, nullptr, D.g);
  CKL();
  D.prof.end(PH_NUMERIC_TOTAL, st);
}

// Coarse matrix (assembled from the local coarse matrices in a fixed order),
// its block factor (right-looking for the symmetric case) and explicit
// inverse, in precision TC.  Returns false if the symmetric factorisation met a
// non-positive pivot.
template <typename TC>
static bool coarse_factor(Device& D, int nc_g, int nbc, const int* dcptr, const long long* dcontrib,
                          vector<void*>& own) {
  cudaStream_t st = D.st;
  BandDesc cb{nbc, nbc - 1, D.ldc, 0, 0, (long long)nbc * nbc * NB * NB,
              (long long)nbc * nbc * NB * NB + (long long)nbc * NB * NB};
  size_t csize = (size_t)cb.oB + (size_t)D.ldc * D.ldc;
  BandDesc cbu = cb;  // U^T band of a general coarse matrix, after the identity block
  if (D.general) {
    cbu.oL = (long long)csize;
    cbu.oLinv = cbu.oL + (long long)nbc * nbc * NB * NB;
    csize = (size_t)cbu.oLinv + (size_t)nbc * NB * NB;
  }
  TC* cpool = dalloc<TC>(csize, own);
  CK(cudaMemsetAsync(cpool, 0, csize * sizeof(TC), st));
  vector<BandDesc> hcbu{cbu};
  BandDesc* dcbu = D.general ? upload(hcbu, own, st) : nullptr;
  if (nc_g > 0) {
    k_coarse_assemble<TC><<<nc_g, 128, 0, st>>>(nc_g, D.ac_ptr, D.ac_col, dcptr, dcontrib, D.small, D.ac_val, cpool,
                                                cb, dcbu);
    CKL();
  }
  k_coarse_pad<TC><<<(D.ldc + 255) / 256, 256, 0, st>>>(nc_g, D.ldc, cpool, cb);
  CKL();
  vector<BandDesc> hcb{cb};
  BandDesc* dcb = upload(hcb, own, st);
  if (D.general) {
    run_factor_lu<TC>(D, dcb, dcbu, 1, nbc, nbc - 1, cpool);
  } else {
    int* cerr = dalloc<int>(1, own);
    CK(cudaMemsetAsync(cerr, 0, sizeof(int), st));
    run_factor_rl<TC>(D, dcb, 1, nbc, nbc - 1, cpool, cerr);
    int herr = 0;
    CK(cudaMemcpyAsync(&herr, cerr, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (herr) return false;
  }
  if constexpr (std::is_same_v<TC, float>) {
    // identity right-hand side needs a column count that is a multiple of the MMA tile
    vector<TcDesc> htc{TcDesc{nbc, nbc - 1, D.ldc, D.ldc, cb.oB, 0, (long long)nbc * nbc * 2 * TC_PCHUNK, -1}};
    TcDesc* tdc = upload(htc, own, st);
    float* cpan = dalloc<float>((size_t)2 * nbc * nbc * 2 * TC_PCHUNK, own);
    run_panels(D, dcb, tdc, 1, nbc, nbc - 1, cpool, cpan, dcbu);
    run_solve_tc(D, tdc, 1, nbc, D.ldc, cpan, cpool);
  } else {
    run_solve<TC>(D, dcb, 1, nbc, D.ldc, cpool, cpool, dcbu);
  }
  D.cinv = cpool + cb.oB;
  return true;
}

// The constraint-dependent part of the setup: Srho factor, [Srho^-1 | Y], G^-1,
// Phi, Z, the local coarse matrices and the coarse problem.  Run after
// setup_numeric, and again when adaptive constraints have changed C; each run
// frees the previous one's buffers.
template <typename T>
static void setup_precond(Solver& S, Device& D) {
  const int nsub = D.nsub;
  cudaStream_t st = D.st;
  D.release_batch();
  D.release_pc();
  auto& own = D.owned_pc;
  long long oP = 0, oPC = 0, oSm = 0, oPan = 0;
  vector<std::array<long long, 2>> poff(nsub, {0, 0});
  int cptr = 0, coff = 0, maxnbi = 0, maxNRC = 0, maxnc = 0;
  D.ncpmax = 4;
  for (int t = 0; t < nsub; ++t) {
    auto& s = S.subs[t];
    if (s.nconstr > 119) throw Error{ERR_UNSUPPORTED, "more than 119 constraints on a subdomain"};
    DevSub& d = D.hs[t];
    d.nc = s.nconstr;
    d.ncp = roundup(std::max(1, d.nc), 4);
    d.NRC = roundup(d.NI + std::max(1, d.nc), TC_M);
    d.oLs = oP; oP += (long long)d.nbi * d.nbi * NB * NB;
    d.oLsinv = oP; oP += (long long)d.nbi * NB * NB;
    d.oBs = oP; oP += (long long)d.NI * d.NRC;
    if (D.general) {
      d.oLsU = oP; oP += (long long)d.nbi * d.nbi * NB * NB;
      d.oLsUinv = oP; oP += (long long)d.nbi * NB * NB;
      d.oYd = oP; oP += (long long)d.NI * d.ncp;
    }
    if (std::is_same_v<T, float>) {
      poff[t][0] = oPan; oPan += (long long)d.nbi * d.nbi * 2 * TC_PCHUNK;
      poff[t][1] = oPan; oPan += (long long)d.nbi * d.nbi * 2 * TC_PCHUNK;
    }
    d.oZ = oPC; oPC += (long long)d.NI * d.NI;
    d.oPhi = oPC; oPC += (long long)d.NI * d.ncp;
    d.oPhid = d.oPhi;
    if (D.general) { d.oPhid = oPC; oPC += (long long)d.NI * d.ncp; }
    d.oGinv = oSm; oSm += (long long)d.ncp * d.ncp;
    d.oAc = oSm; oSm += (long long)d.ncp * d.ncp;
    d.cptr = cptr; cptr += d.nc + 1;
    d.coff = coff; coff += d.nc;
    D.ncpmax = std::max(D.ncpmax, d.ncp);
    maxnbi = std::max(maxnbi, d.nbi); maxNRC = std::max(maxNRC, d.NRC); maxnc = std::max(maxnc, d.nc);
  }
  S.stats.flop_sweep_s = S.stats.bytes_pc_local = 0;
  for (auto& d : D.hs) {
    S.stats.flop_sweep_s += band_sweep_flop(d.nbi, d.nbi - 1, d.NRC, d.NI, !D.general);
    S.stats.bytes_pc_local += (double)d.ni * d.NI * sizeof(T) + (double)d.ni * d.ncp * sizeof(T) + d.ni * 24.0;
  }
  // interface kernels, per launch (each entry read or written once):
  //   assemble_dot: per replicated dof its value and owner record (rep index), per
  //     unique dof the owner pointer, the fixed flag, the weight sum, the dot vector
  //     and the result;
  //   assemble_z: per replicated dof z_s, w_s, its row of Phi (ncp entries), the
  //     weighted correction written and read back with its owner index, the
  //     coarse map per constraint; per unique dof the owner pointer, r, the
  //     weight sum and the result;
  //   coarse_apply: the coarse partials of every subdomain row block, the explicit
  //     inverse three times and the sparse coarse matrix twice.
  {
    double nrep = 0, zrow = 0, nnzc = 0;
    for (auto& d : D.hs) {
      nrep += d.ni;
      zrow += (double)d.ni * ((double)d.ncp * sizeof(T) + 4.0 * d.nc / std::max(1, d.ni));
    }
    const double n = D.n;
    S.stats.bytes_assemble_dot = nrep * (8.0 + 4.0) + n * (4.0 + 4.0 + 8.0 + 8.0 + 8.0);
    S.stats.bytes_assemble_z = nrep * (8.0 + 8.0 + 8.0 + 4.0 + 8.0) + zrow + n * (4.0 + 8.0 + 8.0 + 8.0);
    (void)nnzc;
  }
  T* poolP = dalloc<T>(oP, own);
  D.poolP = poolP;
  float* ppool = std::is_same_v<T, float> ? dalloc<float>(oPan, own) : nullptr;
  D.poolPC = dalloc<T>(oPC, own);
  T* poolPC = static_cast<T*>(D.poolPC);
  D.small = dalloc<double>(oSm, own);
  CK(cudaMemsetAsync(poolP, 0, oP * sizeof(T), st));
  D.ds = upload(D.hs, own, st);
  {
    vector<int> cp, cc, cm;
    vector<double> cv;
    for (int t = 0; t < nsub; ++t) {
      auto& s = S.subs[t];
      int base = (int)cc.size();
      for (int q = 0; q <= s.nconstr; ++q) cp.push_back(base + s.c_ptr[q]);
      cc.insert(cc.end(), s.c_col.begin(), s.c_col.end());
      cv.insert(cv.end(), s.c_val.begin(), s.c_val.end());
      cm.insert(cm.end(), s.indrowc.begin(), s.indrowc.end());
    }
    D.c_ptr = upload(cp, own, st);
    D.c_col = upload(cc, own, st);
    D.c_val = upload(cv, own, st);
    D.cmap = upload(cm, own, st);
    // coarse dof owners
    D.ndofc = S.ndofc;
    vector<int> cptrv(D.ndofc + 1, 0), csub, cloc;
    for (int t = 0; t < nsub; ++t) for (int q : S.subs[t].indrowc) cptrv[q + 1]++;
    for (int q = 0; q < D.ndofc; ++q) cptrv[q + 1] += cptrv[q];
    csub.resize(cptrv[D.ndofc]); cloc.resize(cptrv[D.ndofc]);
    vector<int> cpos(cptrv.begin(), cptrv.end() - 1);
    for (int t = 0; t < nsub; ++t)
      for (int c = 0; c < S.subs[t].nconstr; ++c) {
        int q = S.subs[t].indrowc[c];
        csub[cpos[q]] = t; cloc[cpos[q]++] = c;
      }
    D.co_ptr = upload(cptrv, own, st);
    D.co_sub = upload(csub, own, st);
    D.co_loc = upload(cloc, own, st);
  }
  D.rcpart = dalloc<double>((size_t)nsub * D.nrb * D.ncpmax, own);
  CK(cudaMemsetAsync(D.rcpart, 0, (size_t)nsub * D.nrb * D.ncpmax * sizeof(double), st));
  D.rc = dalloc<double>(std::max(1, D.ndofc), own);
  D.uc = dalloc<double>(std::max(1, D.ndofc), own);
  D.prof.begin(PH_NUMERIC_TOTAL, st, true);
  // ---- preconditioner blocks: Srho factor, [Srho^-1 | Y], G^-1, Phi, Z, local coarse matrices
  vector<BandDesc> hbs(nsub);
  for (int t = 0; t < nsub; ++t) {
    auto& d = D.hs[t];
    hbs[t] = BandDesc{d.nbi, d.nbi - 1, d.NRC, 0, d.oLs, d.oLsinv, d.oBs};
  }
  BandDesc* bd_s = upload(hbs, own, st);
  BandDesc* bdu_s = nullptr;  // U^T band of the general Srho factor
  if (D.general) {
    vector<BandDesc> hbu = hbs;
    for (int t = 0; t < nsub; ++t) { hbu[t].oL = D.hs[t].oLsU; hbu[t].oLinv = D.hs[t].oLsUinv; }
    bdu_s = upload(hbu, own, st);
  }
  D.prof.begin(PH_SRHO_FACTOR, st);
  if (D.general) {
    if constexpr (std::is_same_v<T, float>)
      k_fill_srho_lu<T, float2><<<dim3(D.maxNI / 16, D.maxNI / 16, nsub), dim3(16, 16), 0, st>>>(
          D.ds, static_cast<const float2*>(D.poolS), poolP, bd_s, bdu_s);
    else
      k_fill_srho_lu<T, double><<<dim3(D.maxNI / 16, D.maxNI / 16, nsub), dim3(16, 16), 0, st>>>(
          D.ds, reinterpret_cast<const double*>(D.poolS), poolP, bd_s, bdu_s);
    CKL();
    if (maxnc > 0) {
      k_add_penalty_lu<T><<<dim3(1, nsub), 256, 0, st>>>(D.ds, D.c_ptr, D.c_col, D.c_val, poolP, bd_s, bdu_s);
      CKL();
    }
    run_factor_lu<T>(D, bd_s, bdu_s, nsub, maxnbi, maxnbi - 1, poolP);
  } else {
    if constexpr (std::is_same_v<T, float>)
      k_fill_srho<T, float2><<<dim3(D.maxNI / 16, D.maxNI / 16, nsub), dim3(16, 16), 0, st>>>(
          D.ds, static_cast<const float2*>(D.poolS), poolP, bd_s);
    else
      k_fill_srho<T, double><<<dim3(D.maxNI / 16, D.maxNI / 16, nsub), dim3(16, 16), 0, st>>>(
          D.ds, reinterpret_cast<const double*>(D.poolS), poolP, bd_s);
    CKL();
    if (maxnc > 0) {
      k_add_penalty<T><<<dim3(1, nsub), 256, 0, st>>>(D.ds, D.c_ptr, D.c_col, D.c_val, poolP, bd_s);
      CKL();
    }
    if constexpr (std::is_same_v<T, float>) run_factor_tc(D, bd_s, hbs, nsub, maxnbi, maxnbi - 1, poolP);
    else run_factor<T>(D, bd_s, nsub, maxnbi, maxnbi - 1, poolP);
  }
  TcDesc* td_s = nullptr;
  if constexpr (std::is_same_v<T, float>) {
    vector<TcDesc> hts(nsub);
    for (int t = 0; t < nsub; ++t) {
      auto& d = D.hs[t];
      // [I | C^T]; Srho^-1 is symmetric, so only its lower triangle is formed
      hts[t] = TcDesc{d.nbi, d.nbi - 1, d.NRC, d.NI, d.oBs, poff[t][0], poff[t][1], -1, D.general ? 0 : 1};
    }
    td_s = upload(hts, own, st);
    run_panels(D, bd_s, td_s, nsub, maxnbi, maxnbi - 1, poolP, ppool, bdu_s);
  }
  D.prof.end(PH_SRHO_FACTOR, st);
  D.prof.begin(PH_SRHO_SOLVE, st);
  k_fill_rhs_srho<T><<<dim3((D.maxNI + 127) / 128, nsub), 128, 0, st>>>(D.ds, D.c_ptr, D.c_col, D.c_val, poolP);
  CKL();
  if constexpr (std::is_same_v<T, float>) run_solve_tc(D, td_s, nsub, maxnbi, maxNRC, ppool, poolP);
  else run_solve<T>(D, bd_s, nsub, maxnbi, maxNRC, poolP, poolP, bdu_s);
  D.prof.end(PH_SRHO_SOLVE, st);
  D.prof.begin(PH_PC_BLOCKS, st);
  const int gen = D.general ? 1 : 0;
  if (gen) {  // Y_dual = Srho^-T C^T for the dual coarse basis
    k_ydual<T><<<dim3((D.maxNI * D.ncpmax + 255) / 256, nsub), 256, 0, st>>>(D.ds, D.c_ptr, D.c_col, D.c_val, poolP);
    CKL();
  }
  {
    size_t smem = 2 * (size_t)std::max(1, maxnc) * std::max(1, maxnc) * sizeof(double);
    raise_smem(k_small_g<T>, smem);
    k_small_g<T><<<nsub, 256, smem, st>>>(D.ds, D.c_ptr, D.c_col, D.c_val, poolP, D.small, D.err, gen);
    CKL();
  }
  k_phi<T><<<dim3((D.maxNI * D.ncpmax + 255) / 256, nsub), 256, 0, st>>>(D.ds, poolP, D.small, poolPC, 0);
  CKL();
  if (gen) {
    k_phi<T><<<dim3((D.maxNI * D.ncpmax + 255) / 256, nsub), 256, 0, st>>>(D.ds, poolP, D.small, poolPC, 1);
    CKL();
  }
  if (gen) {
    k_z<T><<<dim3(D.maxNI / 16, D.maxNI / 16, nsub), dim3(16, 16), 0, st>>>(D.ds, poolP, poolPC, gen);
  } else {  // Z and its symmetrisation in one pass
    const size_t zsm = (size_t)4 * 32 * (D.ncpmax + 1) * sizeof(T);
    raise_smem(k_z_sym<T>, zsm);
    k_z_sym<T><<<dim3(D.maxNI / 32, D.maxNI / 32, nsub), dim3(32, 8), zsm, st>>>(D.ds, poolP, poolPC, D.ncpmax);
  }
  CKL();
  D.prof.end(PH_PC_BLOCKS, st);
  D.prof.begin(PH_COARSE, st);

  // ---- coarse problem (levels_prepare_last_level, module_levels.f90:3001-3170):
  // sparse FP64 matrix assembled on the device in a fixed order, factor and
  // explicit inverse in factor precision; the solve is refined in FP64.
  if (S.prm.nlevels == 3) {  // the coarse problem is the level-2 problem (setup_level2)
    D.cres = dalloc<double>(std::max(1, D.ndofc), own);
  } else {
    int nc_g = D.ndofc;
    int nbc = std::max(2, (nc_g + TC_M - 1) / TC_M * 2);  // even number of 64-blocks: ld multiple of 128
    D.ldc = nbc * NB;
    // sparsity and contribution lists (integer work only)
    vector<std::array<long long, 3>> ent;  // (row, col, contribution index)
    for (int t = 0; t < nsub; ++t) {
      auto& sb = S.subs[t];
      auto& d = D.hs[t];
      for (int a = 0; a < d.nc; ++a)
        for (int b2 = 0; b2 < d.nc; ++b2)
          ent.push_back({(long long)sb.indrowc[a], (long long)sb.indrowc[b2], d.oAc + (long long)a * d.ncp + b2});
    }
    std::sort(ent.begin(), ent.end());
    vector<int> aptr(nc_g + 1, 0), acol, acptr(1, 0);
    vector<long long> acontrib;
    for (size_t k = 0; k < ent.size(); ++k) {
      bool fresh = k == 0 || ent[k][0] != ent[k - 1][0] || ent[k][1] != ent[k - 1][1];
      if (fresh) {
        if (k) acptr.push_back((int)acontrib.size());
        acol.push_back((int)ent[k][1]);
        aptr[ent[k][0] + 1]++;
      }
      acontrib.push_back(ent[k][2]);
    }
    acptr.push_back((int)acontrib.size());
    for (int q = 0; q < nc_g; ++q) aptr[q + 1] += aptr[q];
    D.ac_ptr = upload(aptr, own, st);
    D.ac_col = upload(acol, own, st);
    int* dcptr = upload(acptr, own, st);
    long long* dcontrib = upload(acontrib, own, st);
    D.ac_val = dalloc<double>(acol.size(), own);
    // factor and explicit inverse in factor precision; an FP32 factorisation
    // that meets a non-positive pivot (a coarse problem too ill-conditioned
    // for FP32) is redone in FP64.  Very stiff interiors (first refinement
    // ratio above 1e-4: elasticity with stiff inclusions, 6.8e-4) take the FP64
    // route at once: their FP32 coarse data loses accuracy even when the FP32
    // factorisation goes through (two-level 48^3 elasticity: 238 iterations
    // against 226 with the FP64 route, 222 in FP64).  Milder contrast (the
    // channel problem, 3.4e-5) keeps the FP32 coarse factor.
    D.coarse64 = false;
    const bool stiff = std::is_same_v<T, float> && D.refine_r1 > 1e-4f;
    const bool factored = !stiff && coarse_factor<T>(D, nc_g, nbc, dcptr, dcontrib, own);
    if (!factored && !std::is_same_v<T, float>)
      throw Error{ERR_NUMERIC, "non-positive pivot in the FP64 coarse factorisation"};
    if (!factored) {
      // The local coarse matrices G^-1 - rho D^2 come from FP32 factors and can
      // lose their small eigenvalues to cancellation on ill-conditioned
      // subdomains: take Phi^T S Phi with FP64-accurate products instead
      // (the Galerkin form the level-2 problem also uses), and factor in FP64.
      D.coarse64 = true;
      vector<int> all(nsub);
      std::iota(all.begin(), all.end(), 0);
      vector<vector<double>> acs = coarse_energies<T>(D, all, nullptr);
      long long nsm = 0;
      for (auto& d : D.hs) nsm = std::max(nsm, d.oAc + (long long)d.ncp * d.ncp);
      vector<double> hsmall(std::max<long long>(1, nsm));
      CK(cudaMemcpyAsync(hsmall.data(), D.small, nsm * sizeof(double), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      for (int t = 0; t < nsub; ++t) {
        const DevSub& d = D.hs[t];
        for (int r = 0; r < d.nc; ++r)
          for (int c = 0; c < d.nc; ++c) {  // symmetric part
            const double v = 0.5 * (acs[t][(size_t)r * d.nc + c] + acs[t][(size_t)c * d.nc + r]);
            hsmall[d.oAc + (long long)r * d.ncp + c] = v;
          }
      }
      CK(cudaMemcpyAsync(D.small, hsmall.data(), nsm * sizeof(double), cudaMemcpyHostToDevice, st));
      CK(cudaStreamSynchronize(st));
      if (!coarse_factor<double>(D, nc_g, nbc, dcptr, dcontrib, own))
        throw Error{ERR_NUMERIC, "non-positive pivot in the FP64 coarse factorisation"};
    }
    D.cres = dalloc<double>(std::max(1, nc_g), own);
    D.cvdf = dalloc<float2>(std::max(1, nc_g), own);
    {
      double parts = 0;
      for (auto& d : D.hs) parts += (double)D.nrb * d.nc;
      const double esz = D.coarse64 ? 8.0 : (double)sizeof(T);
      S.stats.bytes_coarse_apply = parts * 8.0 + 3.0 * (double)nc_g * nc_g * esz +
                                   2.0 * (double)acol.size() * 12.0 + 8.0 * nc_g * 8.0;
    }
  }
  D.prof.end(PH_COARSE, st);
  D.prof.end(PH_NUMERIC_TOTAL, st);
  CK(cudaStreamSynchronize(st));
}

// Phi_s^T S_s Phi_s for the subdomains in `subs` (nc x nc, row-major), with
// FP64-accurate S products (double-float on the float2 S in mixed precision);
// Phi_s (ni x nc, column-major, FP64) returned in *phis when asked.  The setup's
// local coarse matrices G^-1 - rho D^2 carry the FP32 error of the factors.
template <typename T>
static vector<vector<double>> coarse_energies(Device& D, const vector<int>& subs, vector<vector<double>>* phis) {
  cudaStream_t st = D.st;
  const int nsub = D.nsub;
  vector<vector<double>> out(subs.size());
  if (phis) phis->assign(subs.size(), {});
  if (subs.empty()) return out;
  std::vector<void*> tmp;
  vector<long long> off(subs.size() + 1, 0);
  for (size_t f = 0; f < subs.size(); ++f) off[f + 1] = off[f] + (long long)D.hs[subs[f]].ni * D.hs[subs[f]].nc;
  const long long tot = off[subs.size()];
  vector<double> hphi(std::max<long long>(1, tot));
  {
    vector<T> phi;
    for (size_t f = 0; f < subs.size(); ++f) {
      const DevSub& d = D.hs[subs[f]];
      phi.resize((size_t)d.NI * d.ncp);
      CK(cudaMemcpyAsync(phi.data(), static_cast<const T*>(D.poolPC) + d.oPhi, phi.size() * sizeof(T),
                         cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      for (int c = 0; c < d.nc; ++c)
        for (int r = 0; r < d.ni; ++r) hphi[off[f] + (long long)c * d.ni + r] = (double)phi[(size_t)r * d.ncp + c];
    }
  }
  double* buf = dalloc<double>((size_t)2 * std::max<long long>(1, tot), tmp);
  CK(cudaMemcpyAsync(buf, hphi.data(), tot * sizeof(double), cudaMemcpyHostToDevice, st));
  vector<int> tptr(nsub + 1, 0);
  vector<long long> tin, tout;
  int maxc = 0;
  {
    size_t f = 0;
    vector<int> order(subs.size());
    for (int t = 0; t < nsub; ++t) {
      while (f < subs.size() && subs[f] == t) {
        const DevSub& d = D.hs[t];
        for (int c = 0; c < d.nc; ++c) {
          tin.push_back(off[f] + (long long)c * d.ni);
          tout.push_back(tot + off[f] + (long long)c * d.ni);
        }
        maxc = std::max(maxc, d.nc);
        ++f;
      }
      tptr[t + 1] = (int)tin.size();
    }
  }
  ColTab tab{upload(tptr, tmp, st), upload(tin, tmp, st), upload(tout, tmp, st)};
  dim3 g((D.maxNI + 63) / 64, (maxc + 63) / 64, nsub);
  if (D.mixed) k_ad_gemm_df<<<g, 256, 0, st>>>(D.ds, static_cast<const float2*>(D.poolS), tab, buf);
  else k_ad_gemm<double, false, double><<<g, 256, 0, st>>>(D.ds, static_cast<const double*>(D.poolS), tab, buf);
  CKL();
  vector<double> hsphi(std::max<long long>(1, tot));
  CK(cudaMemcpyAsync(hsphi.data(), buf + tot, tot * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (void* q : tmp) cudaFreeAsync(q, st);
#pragma omp parallel for schedule(dynamic)
  for (int f = 0; f < (int)subs.size(); ++f) {
    const DevSub& d = D.hs[subs[f]];
    const double* ph = &hphi[off[f]];
    const double* sp = &hsphi[off[f]];
    vector<double>& ac = out[f];
    ac.assign((size_t)d.nc * d.nc, 0.0);
    for (int a = 0; a < d.nc; ++a)
      for (int b = 0; b < d.nc; ++b) {
        double t2 = 0.0;
        for (int r = 0; r < d.ni; ++r) t2 += ph[(long long)a * d.ni + r] * sp[(long long)b * d.ni + r];
        ac[(size_t)a * d.nc + b] = t2;
      }
  }
  if (phis)
    for (size_t f = 0; f < subs.size(); ++f) (*phis)[f].assign(hphi.begin() + off[f], hphi.begin() + off[f + 1]);
  return out;
}

// ------------------------------------------------------------ adaptive constraints
// Batched LOBPCG over all face pairs (adaptivity_solve_eigenvectors,
// module_adaptivity.f90:296-2514; 15 iterations as lobpcg_maxit, :38), then
// the eigenvectors above the threshold become face constraints
// (host_load_adaptive).  Uses S and the subdomain corrections Z of the
// preconditioner built from the standard constraints.
template <typename T>
static void adaptive_constraints(Solver& S, Device& D) {
  const double t0 = wall_time();
  cudaStream_t st = D.st;
  D.prof.begin(PH_NUMERIC_TOTAL, st, true);  // part of the device setup time
  // null spaces of the floating subdomains' Schur complements: Phi y for the
  // null vectors y of Phi^T S Phi, formed with FP64-accurate S products (the
  // null-space projection of module_adaptivity.f90:1180-1480, per subdomain)
  const int nsub = D.nsub;
  vector<vector<double>> nulls(nsub);
  {
    vector<int> fl;
    for (int t = 0; t < nsub; ++t)
      if (!S.subs[t].bc_present && D.hs[t].nc > 0) fl.push_back(t);
    vector<vector<double>> phis;
    vector<vector<double>> acs = coarse_energies<T>(D, fl, &phis);
#pragma omp parallel for schedule(dynamic)
    for (int f = 0; f < (int)fl.size(); ++f) {
      const DevSub& d = D.hs[fl[f]];
      const double* ph = phis[f].data();
      int dn = 0;
      vector<double> y = host_coarse_null_coefficients(d.nc, d.nc, acs[f].data(), dn);
      vector<double>& nv = nulls[fl[f]];
      nv.assign((size_t)d.ni * dn, 0.0);
      for (int c = 0; c < dn; ++c) {
        for (int r = 0; r < d.ni; ++r) {
          double acc = 0.0;
          for (int q = 0; q < d.nc; ++q) acc += ph[(long long)q * d.ni + r] * y[(size_t)q * dn + c];
          nv[(size_t)c * d.ni + r] = acc;
        }
        for (int pass = 0; pass < 2; ++pass)
          for (int c2 = 0; c2 < c; ++c2) {
            double tt = 0.0;
            for (int r = 0; r < d.ni; ++r) tt += nv[(size_t)c2 * d.ni + r] * nv[(size_t)c * d.ni + r];
            for (int r = 0; r < d.ni; ++r) nv[(size_t)c * d.ni + r] -= tt * nv[(size_t)c2 * d.ni + r];
          }
        double nn = 0.0;
        for (int r = 0; r < d.ni; ++r) nn += nv[(size_t)c * d.ni + r] * nv[(size_t)c * d.ni + r];
        nn = std::sqrt(nn);
        for (int r = 0; r < d.ni; ++r) nv[(size_t)c * d.ni + r] = nn > 0 ? nv[(size_t)c * d.ni + r] / nn : 0.0;
      }
    }
  }
  AdaptivePairs P;
  host_adaptive_pairs(S, P, nulls);
  S.stats.npair = P.npair;
  const int np = P.npair;
  vector<double> eig((size_t)std::max(1, np) * AD_KM, 0.0), cons;
  if (np > 0) {
    std::vector<void*> tmp;  // freed at the end of this step
    vector<PairDev> hp(np);
    for (int p = 0; p < np; ++p) {
      if (P.m[p] > AD_MAXM) throw Error{ERR_UNSUPPORTED, "more than 48 coarse dofs shared by a face pair"};
      hp[p] = PairDev{P.si[p], P.sj[p], P.ni[p], P.n[p], P.m[p], P.k[p], P.cptr[p], P.cptr[p + 1], P.vo[p], P.qo[p]};
    }
    PairDev* pd = upload(hp, tmp, st);
    double* dq = upload(P.q, tmp, st);
    int* dca = upload(P.ca, tmp, st);
    int* dcb = upload(P.cb, tmp, st);
    double* dwa = upload(P.wa, tmp, st);
    double* dwb = upload(P.wb, tmp, st);
    const long long nvec = P.nvec;
    double* va = dalloc<double>((size_t)AB_NBLK * nvec, tmp);
    CK(cudaMemsetAsync(va, 0, (size_t)AB_NBLK * nvec * sizeof(double), st));
    double* G = dalloc<double>((size_t)np * 2 * AD_NB * AD_NB, tmp);
    CK(cudaMemsetAsync(G, 0, (size_t)np * 2 * AD_NB * AD_NB * sizeof(double), st));
    double* C = dalloc<double>((size_t)np * AD_NB * AD_KM, tmp);
    double* lam = dalloc<double>((size_t)np * AD_KM, tmp);
    CK(cudaMemsetAsync(lam, 0, (size_t)np * AD_KM * sizeof(double), st));
    // pair coarse problems for the preconditioner: K = assembled Phi^T S Phi of
    // both subdomains over the union of their coarse dofs, regularised along
    // the coarse values of null(S) within null(D), inverted on the host
    vector<int> hnu(np), hmofs(np), hmap;
    vector<long long> hkofs(np);
    vector<double> hkinv;
    {
      long long nsm = 0;
      for (auto& d : D.hs) nsm = std::max(nsm, d.oAc + (long long)d.ncp * d.ncp);
      vector<double> hsmall(std::max<long long>(1, nsm));
      CK(cudaMemcpyAsync(hsmall.data(), D.small, nsm * sizeof(double), cudaMemcpyDeviceToHost, st));
      CK(cudaStreamSynchronize(st));
      vector<vector<int>> maps(np);
      vector<vector<double>> kinv(np);
      std::string errs;
#pragma omp parallel for schedule(dynamic)
      for (int p = 0; p < np; ++p) {
        const Subdomain& A = S.subs[P.si[p]];
        const Subdomain& Bs = S.subs[P.sj[p]];
        const DevSub& di = D.hs[P.si[p]];
        const DevSub& dj = D.hs[P.sj[p]];
        std::unordered_map<int, int> pos;
        vector<int>& mp = maps[p];
        int nu = 0;
        for (int qq = 0; qq < A.nconstr; ++qq) { pos[A.indrowc[qq]] = nu; mp.push_back(nu++); }
        for (int qq = 0; qq < Bs.nconstr; ++qq) {
          auto it = pos.find(Bs.indrowc[qq]);
          if (it != pos.end()) mp.push_back(it->second);
          else { pos[Bs.indrowc[qq]] = nu; mp.push_back(nu++); }
        }
        hnu[p] = nu;
        if (nu > AD_NUMAX) {
#pragma omp critical
          errs = "more than 256 coarse dofs in a face pair";
          continue;
        }
        vector<double> K((size_t)nu * nu, 0.0);
        for (int a = 0; a < A.nconstr; ++a)
          for (int b = 0; b < A.nconstr; ++b) K[(size_t)mp[a] * nu + mp[b]] += hsmall[di.oAc + (long long)a * di.ncp + b];
        for (int a = 0; a < Bs.nconstr; ++a)
          for (int b = 0; b < Bs.nconstr; ++b)
            K[(size_t)mp[A.nconstr + a] * nu + mp[A.nconstr + b]] += hsmall[dj.oAc + (long long)a * dj.ncp + b];
        double kmax = 0.0;
        for (int a = 0; a < nu; ++a) kmax = std::max(kmax, K[(size_t)a * nu + a]);
        for (int c = P.md[p]; c < P.m[p]; ++c) {  // coarse values y = C v of the null directions
          const double* v = &P.q[P.qo[p] + (long long)c * P.n[p]];
          vector<double> y(nu, 0.0);
          for (int r = 0; r < A.nconstr; ++r) {
            double t = 0.0;
            for (int e = A.c_ptr[r]; e < A.c_ptr[r + 1]; ++e) t += A.c_val[e] * v[A.c_col[e]];
            y[mp[r]] = t;
          }
          for (int r = 0; r < Bs.nconstr; ++r) {
            double t = 0.0;
            for (int e = Bs.c_ptr[r]; e < Bs.c_ptr[r + 1]; ++e) t += Bs.c_val[e] * v[P.ni[p] + Bs.c_col[e]];
            y[mp[A.nconstr + r]] = t;
          }
          double yy = 0.0;
          for (double x : y) yy += x * x;
          if (yy > 0)
            for (int a = 0; a < nu; ++a)
              for (int b = 0; b < nu; ++b) K[(size_t)a * nu + b] += kmax * y[a] * y[b] / yy;
        }
        // Cholesky, then the explicit inverse
        vector<double> L = K;
        bool ok = true;
        for (int j = 0; j < nu && ok; ++j) {
          double sum = L[(size_t)j * nu + j];
          for (int t = 0; t < j; ++t) sum -= L[(size_t)j * nu + t] * L[(size_t)j * nu + t];
          if (!(sum > 1e-14 * kmax)) { ok = false; break; }
          const double dj2 = std::sqrt(sum);
          L[(size_t)j * nu + j] = dj2;
          for (int i = j + 1; i < nu; ++i) {
            double t = L[(size_t)i * nu + j];
            for (int k2 = 0; k2 < j; ++k2) t -= L[(size_t)i * nu + k2] * L[(size_t)j * nu + k2];
            L[(size_t)i * nu + j] = t / dj2;
          }
        }
        vector<double>& Ki = kinv[p];
        Ki.assign((size_t)nu * nu, 0.0);
        if (!ok) continue;  // singular pair coarse problem: no coarse correction for this pair
        for (int c = 0; c < nu; ++c) {
          vector<double> x(nu, 0.0);
          x[c] = 1.0;
          for (int i = 0; i < nu; ++i) {
            double t = x[i];
            for (int k2 = 0; k2 < i; ++k2) t -= L[(size_t)i * nu + k2] * x[k2];
            x[i] = t / L[(size_t)i * nu + i];
          }
          for (int i = nu - 1; i >= 0; --i) {
            double t = x[i];
            for (int k2 = i + 1; k2 < nu; ++k2) t -= L[(size_t)k2 * nu + i] * x[k2];
            x[i] = t / L[(size_t)i * nu + i];
          }
          for (int i = 0; i < nu; ++i) Ki[(size_t)i * nu + c] = x[i];
        }
      }
      if (!errs.empty()) throw Error{ERR_UNSUPPORTED, errs};
      long long ko = 0;
      for (int p = 0; p < np; ++p) {
        hmofs[p] = (int)hmap.size();
        hmap.insert(hmap.end(), maps[p].begin(), maps[p].end());
        hkofs[p] = ko;
        ko += (long long)hnu[p] * hnu[p];
        hkinv.insert(hkinv.end(), kinv[p].begin(), kinv[p].end());
      }
    }
    PairCoarse pcoarse{upload(hnu, tmp, st), upload(hmofs, tmp, st), upload(hmap, tmp, st), upload(hkofs, tmp, st),
                       upload(hkinv, tmp, st)};
    // column tables of the batched products: per subdomain, every pair column it takes part in
    struct Tab { vector<int> ptr; vector<long long> in, out; int maxc = 0; ColTab dev{}; };
    auto build = [&](std::initializer_list<std::pair<int, int>> io) {
      Tab t;
      vector<vector<long long>> in(nsub), out(nsub);
      for (int p = 0; p < np; ++p)
        for (int side = 0; side < 2; ++side) {
          const int sub = side == 0 ? P.si[p] : P.sj[p];
          const long long roff = side == 0 ? 0 : P.ni[p];
          for (auto& pr : io)
            for (int c = 0; c < P.k[p]; ++c) {
              in[sub].push_back(pr.first * nvec + P.vo[p] + (long long)c * P.n[p] + roff);
              out[sub].push_back(pr.second * nvec + P.vo[p] + (long long)c * P.n[p] + roff);
            }
        }
      t.ptr.assign(nsub + 1, 0);
      for (int s2 = 0; s2 < nsub; ++s2) {
        t.ptr[s2 + 1] = t.ptr[s2] + (int)in[s2].size();
        t.maxc = std::max(t.maxc, (int)in[s2].size());
        t.in.insert(t.in.end(), in[s2].begin(), in[s2].end());
        t.out.insert(t.out.end(), out[s2].begin(), out[s2].end());
      }
      t.dev.ptr = upload(t.ptr, tmp, st);
      t.dev.in = upload(t.in, tmp, st);
      t.dev.out = upload(t.out, tmp, st);
      return t;
    };
    Tab tabX = build({{AB_T1, AB_T2}, {AB_X, AB_BX}});
    Tab tabW = build({{AB_T1, AB_T2}, {AB_W, AB_BW}});
    Tab tabZ = build({{AB_T1, AB_W}});
    int maxn = 0;
    for (int p = 0; p < np; ++p) maxn = std::max(maxn, P.n[p]);
    const dim3 gpair(np);
    auto gemm_s = [&](const Tab& t) {
      if (t.maxc == 0) return;
      dim3 g((D.maxNI + 63) / 64, (t.maxc + 63) / 64, nsub);
      if (D.mixed)
        k_ad_gemm_df<<<g, 256, 0, st>>>(D.ds, static_cast<const float2*>(D.poolS), t.dev, va);
      else
        k_ad_gemm<double, false, double><<<g, 256, 0, st>>>(D.ds, static_cast<const double*>(D.poolS), t.dev, va);
      CKL();
    };
    auto project = [&](int b0, int b1) {
      k_ad_project<<<dim3(np, b1 >= 0 ? 2 : 1), 256, 0, st>>>(pd, dq, va, nvec, b0, b1);
      CKL();
    };
    // (A b, B b) for a projected block b (X or W)
    auto apply_ab = [&](int b, int ab, int bb, const Tab& t) {
      (void)bb;
      k_ad_ire<<<gpair, 256, 0, st>>>(pd, dca, dcb, dwa, dwb, va, nvec, b, AB_T1, 0);
      CKL();
      gemm_s(t);
      k_ad_ire<<<gpair, 256, 0, st>>>(pd, dca, dcb, dwa, dwb, va, nvec, AB_T2, ab, 1);
      CKL();
      project(ab, bb);
    };
    auto rayleigh_ritz = [&](int nb) {
      k_ad_gram<<<dim3(np, 6, 2), 256, 0, st>>>(pd, va, nvec, G, nb);
      CKL();
      k_ad_rr<<<np, 32, 0, st>>>(pd, G, C, lam, nb);
      CKL();
      k_ad_update<<<dim3(np, 3, (maxn + 127) / 128), 128, 0, st>>>(pd, va, nvec, C, nb);
      CKL();
    };
    k_ad_random<<<gpair, 256, 0, st>>>(pd, va, nvec);
    CKL();
    project(AB_X, -1);
    apply_ab(AB_X, AB_AX, AB_BX, tabX);
    rayleigh_ritz(1);
    const int maxit = 15;
    for (int it = 1; it <= maxit; ++it) {
      k_ad_residual<<<dim3(np, (maxn + 255) / 256), 256, 0, st>>>(pd, va, nvec, lam);
      CKL();
      // W = P Z P R
      if (tabZ.maxc > 0) {
        dim3 g((D.maxNI + 63) / 64, (tabZ.maxc + 63) / 64, nsub);
        k_ad_gemm<T, true, float><<<g, 256, 0, st>>>(D.ds, static_cast<const T*>(D.poolPC), tabZ.dev, va);
        CKL();
      }
      k_ad_coarse<T><<<dim3(np, AD_KM), 256, 0, st>>>(pd, pcoarse, D.ds, static_cast<const T*>(D.poolPC), va, nvec);
      CKL();
      project(AB_W, -1);
      apply_ab(AB_W, AB_AW, AB_BW, tabW);
      rayleigh_ritz(it == 1 ? 2 : 3);
    }
    S.stats.lobpcg_iter = maxit;
    double* rn = dalloc<double>((size_t)np * AD_KM, tmp);
    CK(cudaMemsetAsync(rn, 0, (size_t)np * AD_KM * sizeof(double), st));
    k_ad_resnorm<<<dim3(np, AD_KM), 256, 0, st>>>(pd, va, nvec, lam, rn);
    CKL();
    vector<double> hrn((size_t)np * AD_KM);
    CK(cudaMemcpyAsync(eig.data(), lam, eig.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(hrn.data(), rn, hrn.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    S.stats.lobpcg_resid = 0;
    for (int p = 0; p < np; ++p)
      for (int c = 0; c < P.k[p]; ++c)
        if (eig[(size_t)p * AD_KM + c] >= S.prm.adaptive_tau)
          S.stats.lobpcg_resid = std::max(S.stats.lobpcg_resid, hrn[(size_t)p * AD_KM + c]);
    // A x of the selected eigenvectors
    vector<long long> src, dst;
    vector<int> len;
    long long tot = 0;
    double est = -1.0;
    for (int p = 0; p < np; ++p) {
      int nad = 0;
      for (int c = 0; c < P.k[p]; ++c)
        if (eig[(size_t)p * AD_KM + c] >= S.prm.adaptive_tau) {
          src.push_back(AB_AX * nvec + P.vo[p] + (long long)c * P.n[p]);
          dst.push_back(tot);
          len.push_back(P.n[p]);
          tot += P.n[p];
          ++nad;
        }
      // estimate of the condition number (module_adaptivity.f90:2156-2170)
      double el = 1.0;
      if (P.k[p] > 0) el = nad < P.k[p] ? eig[(size_t)p * AD_KM + nad] : eig[(size_t)p * AD_KM + nad - 1];
      est = std::max(est, el);
    }
    S.stats.adapt_est = est;
    cons.assign(std::max<long long>(1, tot), 0.0);
    if (!src.empty()) {
      long long* dsrc = upload(src, tmp, st);
      long long* ddst = upload(dst, tmp, st);
      int* dlen = upload(len, tmp, st);
      double* dout = dalloc<double>((size_t)tot, tmp);
      k_ad_gather<<<(int)src.size(), 256, 0, st>>>(va, dsrc, ddst, dlen, dout);
      CKL();
      CK(cudaMemcpyAsync(cons.data(), dout, (size_t)tot * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    CK(cudaStreamSynchronize(st));
    for (void* q : tmp) cudaFreeAsync(q, st);
  }
  S.adaptive_eigs = eig;
  S.adaptive_pairs = P;
  host_load_adaptive(S, P, eig, cons);
  D.prof.end(PH_NUMERIC_TOTAL, st);
  S.stats.t_adaptive = wall_time() - t0;
}

// ------------------------------------------------------------ PCG driver
template <typename T>
static void launch_schur(Device& D, const double* vin, double* vout, bool zero_fixed, const PcgCtl* ctl,
                         const double* dotvec) {
  dim3 grid(D.nrb, D.nsub);
  D.prof.begin(PH_SCHUR_APPLY, D.st);
  if (D.mixed) {
    size_t smem = (size_t)D.maxNI * sizeof(float2);
    k_schur_apply_df<<<grid, AT, smem, D.st>>>(D.ds, static_cast<const float2*>(D.poolS), vin, D.uniq, D.yrep, ctl);
  } else {
    size_t smem = (size_t)D.maxNI * sizeof(double);
    k_schur_apply_f64<<<grid, AT, smem, D.st>>>(D.ds, static_cast<const double*>(D.poolS), vin, D.uniq, D.yrep, ctl);
  }
  CKL();
  D.prof.end(PH_SCHUR_APPLY, D.st);
  D.prof.begin(PH_ASSEMBLE_DOT, D.st);
  k_assemble_dot<<<D.npart, RT, 0, D.st>>>(D.n, D.own, D.yrep, D.fixed, D.wsum, dotvec, vout, D.part, ctl,
                                           zero_fixed ? 1 : 0);
  CKL();
  D.prof.end(PH_ASSEMBLE_DOT, D.st);
}

static void level2_apply(Device& D1, const double* rc, double* uc);

template <typename T>
static void launch_pc(Device& D, const double* rin, double* zout, const PcgCtl* ctl) {
  dim3 grid(D.nrb, D.nsub);
  size_t smem = (size_t)D.maxNI * sizeof(typename PcVec<T>::type);
  D.prof.begin(PH_PC_LOCAL, D.st);
  k_pc_local<T><<<grid, AT, smem, D.st>>>(D.ds, static_cast<const T*>(D.poolPC), rin, D.uniq, D.wrep, D.zrep,
                                          D.rcpart, D.nrb, D.ncpmax, ctl);
  CKL();
  D.prof.end(PH_PC_LOCAL, D.st);
  if (D.ndofc > 0 && D.lev2) {
    k_coarse_gather<<<(D.ndofc + 255) / 256, 256, 0, D.st>>>(D.ndofc, D.co_ptr, D.co_sub, D.co_loc, D.ds, D.rcpart,
                                                           D.nrb, D.ncpmax, D.rc, ctl);
    CKL();
    level2_apply(D, D.rc, D.uc);
  } else if (D.ndofc > 0) {
    D.prof.begin(PH_COARSE_APPLY, D.st);
    // FP32 inverse: its operand also as double-float pairs (in vdf)
    float2* vdf = (!D.coarse64 && std::is_same_v<T, float>) ? D.cvdf : nullptr;
    k_coarse_gather<<<(D.ndofc + 255) / 256, 256, 0, D.st>>>(D.ndofc, D.co_ptr, D.co_sub, D.co_loc, D.ds, D.rcpart,
                                                           D.nrb, D.ncpmax, D.rc, ctl, vdf);
    CKL();
    int gb = (D.ndofc + 7) / 8;
    auto gemv = [&](const double* v, int mode) {
      if (D.coarse64)
        k_coarse_gemv<double><<<gb, 256, 0, D.st>>>(D.ndofc, D.ldc, static_cast<const double*>(D.cinv), v, nullptr,
                                                     D.uc, mode, ctl);
      else
        k_coarse_gemv<T><<<gb, 256, 0, D.st>>>(D.ndofc, D.ldc, static_cast<const T*>(D.cinv), v, vdf, D.uc, mode,
                                               ctl);
    };
    gemv(D.rc, 0);
    for (int rr = 0; rr < 2; ++rr) {
      k_coarse_residual<<<(D.ndofc + 255) / 256, 256, 0, D.st>>>(D.ndofc, D.ac_ptr, D.ac_col, D.ac_val, D.rc, D.uc,
                                                               D.cres, ctl, vdf);
      gemv(D.cres, 1);
    }
    CKL();
    D.prof.end(PH_COARSE_APPLY, D.st);
  }
  D.prof.begin(PH_ASSEMBLE_Z, D.st);
  const size_t zsm = (size_t)D.ncpmax * sizeof(typename PcVec<T>::type) + (size_t)ZP_ROWS * (D.ncpmax + 1) * sizeof(T);
  if (zsm <= 200 * 1024) {  // weighted corrections per subdomain row, then the sum per unique dof
    raise_smem(k_zphi<T>, zsm);
    k_zphi<T><<<dim3((D.maxNI + ZP_ROWS - 1) / ZP_ROWS, D.nsub), ZP_ROWS, zsm, D.st>>>(
        D.ds, static_cast<const T*>(D.poolPC), D.zrep, D.wrep, D.cmap, D.ndofc > 0 ? D.uc : nullptr, D.zw, ctl);
    CKL();
    k_assemble_dot<<<D.npart, RT, 0, D.st>>>(D.n, D.own, D.zw, D.fixed, D.wsum, rin, zout, D.part, ctl, 0);
  } else {  // very many constraints per subdomain: one pass per unique dof
    k_assemble_z<T><<<D.npart, RT, 0, D.st>>>(D.n, D.own, D.ds, static_cast<const T*>(D.poolPC), D.zrep, D.wrep,
                                              D.cmap, D.uc, D.wsum, rin, zout, D.part, ctl);
  }
  CKL();
  D.prof.end(PH_ASSEMBLE_Z, D.st);
}

static double host_sum_parts(Device& D) {
  k_sum_parts<<<1, RT, 0, D.st>>>(D.part, D.npart, D.scal);
  CKL();
  double v = 0.0;
  CK(cudaMemcpyAsync(&v, D.scal, sizeof(double), cudaMemcpyDeviceToHost, D.st));
  CK(cudaStreamSynchronize(D.st));
  return v;
}

// largest eigenvalue of the Lanczos tridiagonal matrix by Sturm bisection
// (stands in for LAPACK DSTEV in krylov_condsparse, module_krylov.f90:2061-2118)
static double lanczos_max_eig(const vector<double>& d, const vector<double>& e) {
  int n = (int)d.size();
  if (n <= 1) return 1.0;
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < n; ++i) {
    double rr = (i > 0 ? std::fabs(e[i - 1]) : 0.0) + (i < n - 1 ? std::fabs(e[i]) : 0.0);
    lo = std::min(lo, d[i] - rr);
    hi = std::max(hi, d[i] + rr);
  }
  auto below = [&](double xv) {
    int cnt = 0;
    double q = 1.0;
    for (int i = 0; i < n; ++i) {
      q = d[i] - xv - (i > 0 ? e[i - 1] * e[i - 1] / q : 0.0);
      if (q == 0.0) q = -1e-300;
      if (q < 0) cnt++;
    }
    return cnt;
  };
  for (int it = 0; it < 200 && hi - lo > 1e-15 * std::max(1.0, std::fabs(hi)); ++it) {
    double mid = 0.5 * (lo + hi);
    if (below(mid) >= n) hi = mid; else lo = mid;
  }
  return 0.5 * (lo + hi);
}

// BiCGSTAB (method 1, module_krylov.f90:948-1505) and steepest descent
// (method 2, module_krylov.f90:1508-1840) on the interface problem, with the
// same Schur and BDDC operators as PCG.  r holds g - S x0 with the fixed
// dofs zeroed, normrhs its weighted norm (> 0).  Host-driven: each scalar is
// read back once per use.
template <typename T>
static void other_krylov(Solver& S, int method, double normrhs, double tol, int maxit, int ndecrmax, int& num_iter,
                         int& reason) {
  Device& D = *S.dev;
  cudaStream_t st = D.st;
  auto& own = D.owned;
  if (!D.kv) {
    D.kv = dalloc<double>(D.n, own); D.ky = dalloc<double>(D.n, own); D.ks = dalloc<double>(D.n, own);
    D.kt = dalloc<double>(D.n, own); D.krs = dalloc<double>(D.n, own);
  }
  const int nb = (D.n + 255) / 256;
  const size_t bytes = (size_t)D.n * sizeof(double);
  auto dot = [&](const double* a, const double* b) {
    k_dot<<<D.npart, RT, 0, st>>>(D.n, a, b, D.wsum, D.part);
    CKL();
    return host_sum_parts(D);
  };
  auto axpy = [&](double a, const double* x, double* y) {
    k_axpy<<<nb, 256, 0, st>>>(D.n, a, x, y);
    CKL();
  };
  auto copy = [&](const double* x, double* y) { CK(cudaMemcpyAsync(y, x, bytes, cudaMemcpyDeviceToDevice, st)); };
  int ndecr = 0;
  double lastres = 1.0;
  num_iter = 0;
  reason = -1;
  if (method == 2) {  // steepest descent: z = M r, x += alpha z, r -= alpha S z
    for (int iter = 1; iter <= maxit; ++iter) {
      launch_pc<T>(D, D.r, D.z, nullptr);
      launch_schur<T>(D, D.z, D.ap, false, nullptr, nullptr);
      const double alpha = dot(D.r, D.z) / dot(D.z, D.ap);
      axpy(alpha, D.z, D.x);
      axpy(-alpha, D.ap, D.r);
      k_zero_fixed<<<nb, 256, 0, st>>>(D.n, D.fixed, D.r);
      CKL();
      const double relres = std::sqrt(dot(D.r, D.r)) / normrhs;
      S.relres_history.push_back(relres);
      num_iter = iter;
      if (relres < tol) { reason = 0; return; }
      if (iter == maxit) { reason = -1; return; }
      // the reference stops with an error here (module_krylov.f90:1801-1812)
      if (relres < lastres) ndecr = 0;
      else if (++ndecr >= ndecrmax) { reason = -2; return; }
      lastres = relres;
    }
    return;
  }
  // BiCGSTAB with the shadow residual r~ = r0
  double rhoold = 1.0, alpha = 1.0, omega = 1.0;
  CK(cudaMemsetAsync(D.kv, 0, bytes, st));
  CK(cudaMemsetAsync(D.p, 0, bytes, st));
  copy(D.r, D.krs);
  for (int iter = 1; iter <= maxit; ++iter) {
    const double rho = dot(D.r, D.krs);
    const double beta = rho * alpha / (rhoold * omega);
    axpy(-omega, D.kv, D.p);  // p = r + beta (p - omega v)
    k_axpby<<<nb, 256, 0, st>>>(D.n, 1.0, D.r, beta, D.p);
    CKL();
    launch_pc<T>(D, D.p, D.ky, nullptr);                   // y = M p
    launch_schur<T>(D, D.ky, D.kv, false, nullptr, nullptr);  // v = S y
    alpha = rho / dot(D.kv, D.krs);
    axpy(alpha, D.ky, D.x);
    copy(D.r, D.ks);  // s = r - alpha v
    axpy(-alpha, D.kv, D.ks);
    double relres = std::sqrt(dot(D.ks, D.ks)) / normrhs;
    num_iter = iter;
    if (relres < tol) { S.relres_history.push_back(relres); reason = 0; return; }
    if (relres < lastres) ndecr = 0;
    else if (++ndecr >= ndecrmax) { S.relres_history.push_back(relres); reason = -2; return; }
    lastres = relres;
    launch_pc<T>(D, D.ks, D.z, nullptr);                   // z = M s
    launch_schur<T>(D, D.z, D.kt, false, nullptr, nullptr);  // t = S z
    omega = dot(D.kt, D.ks) / dot(D.kt, D.kt);
    axpy(omega, D.z, D.x);
    copy(D.ks, D.r);  // r = s - omega t
    axpy(-omega, D.kt, D.r);
    relres = std::sqrt(dot(D.r, D.r)) / normrhs;
    S.relres_history.push_back(relres);
    if (relres < tol) { reason = 0; return; }
    if (iter == maxit) { reason = -1; return; }
    if (relres < lastres) ndecr = 0;
    else if (++ndecr >= ndecrmax) { reason = -2; return; }
    lastres = relres;
    rhoold = rho;
  }
}

template <typename T>
static bool solve_impl(Solver& S, int method, double tol, int maxit, int ndecrmax, int recycling, int maxvec,
                       int& num_iter, int& reason, double& cond) {
  Device& D = *S.dev;
  cudaStream_t st = D.st;
  auto& own = D.owned;
  double t0 = wall_time();
  if (maxit + 2 > D.maxit_alloc) {
    D.maxit_alloc = maxit + 2;
    D.hist = dalloc<double>(D.maxit_alloc, own);
    D.diag = dalloc<double>(D.maxit_alloc, own);
    D.subdiag = dalloc<double>(D.maxit_alloc, own);
  }
  CK(cudaMemsetAsync(D.diag, 0, D.maxit_alloc * sizeof(double), st));
  CK(cudaMemsetAsync(D.subdiag, 0, D.maxit_alloc * sizeof(double), st));
  // initial guess restricted to the interface with Dirichlet values (module_levels.f90:4374-4440)
  {
    vector<double> x0(D.n, 0.0);
    vector<char> seen(D.n, 0);
    for (auto& s : S.subs)
      for (int i = 0; i < s.ndofi; ++i) {
        int u = s.uniq[i];
        if (seen[u]) continue;
        seen[u] = 1;
        int d = s.iivsvn[i];
        x0[u] = (s.bc_present && s.ifix[d]) ? s.fixv[d] : s.sol[d];
      }
    CK(cudaMemcpyAsync(D.x, x0.data(), D.n * sizeof(double), cudaMemcpyHostToDevice, st));
    g_h2d_bytes += D.n * sizeof(double);
    CK(cudaStreamSynchronize(st));
  }
  long long launches0 = g_launches;
  D.prof.begin(PH_SOLVE_TOTAL, st, true);
  // r = g with fixed interface dofs zeroed (module_krylov.f90:222-236)
  k_assemble_plain<<<(D.n + 255) / 256, 256, 0, st>>>(D.n, D.own, D.grep, D.fixed, D.r);
  CKL();
  num_iter = 0; reason = 0; cond = method == 0 ? 1.0 : -1.0;
  S.relres_history.clear();
  bool postprocess = true;
  bool stalled = false;  // steepest descent without decrease: an error in the reference
  if (method != 0) {
    // BiCGSTAB / steepest descent: normalised by the norm of r = g - S x0
    // (module_krylov.f90:1065-1113, 1620-1662)
    launch_schur<T>(D, D.x, D.ap, true, nullptr, nullptr);
    k_axpy<<<(D.n + 255) / 256, 256, 0, st>>>(D.n, -1.0, D.ap, D.r);
    CKL();
    k_dot<<<D.npart, RT, 0, st>>>(D.n, D.r, D.r, D.wsum, D.part);
    CKL();
    const double normrhs = std::sqrt(host_sum_parts(D));
    if (normrhs == 0.0) {
      postprocess = false;
    } else {
      double tl = wall_time();
      D.prof.begin(PH_PCG, st);
      other_krylov<T>(S, method, normrhs, tol, maxit, ndecrmax, num_iter, reason);
      D.prof.end(PH_PCG, st);
      S.stats.t_iterations = wall_time() - tl;
      stalled = method == 2 && reason == -2;
      if (stalled) postprocess = false;
    }
  }
  double normrhs2 = 0.0;
  if (method == 0) {
    k_dot<<<D.npart, RT, 0, st>>>(D.n, D.r, D.r, D.wsum, D.part);
    CKL();
    normrhs2 = host_sum_parts(D);
    if (normrhs2 == 0.0) postprocess = false;
  }
  if (method == 0 && normrhs2 != 0.0) {
    launch_schur<T>(D, D.x, D.ap, true, nullptr, nullptr);
    k_axpy<<<(D.n + 255) / 256, 256, 0, st>>>(D.n, -1.0, D.ap, D.r);
    CKL();
    k_dot<<<D.npart, RT, 0, st>>>(D.n, D.r, D.r, D.wsum, D.part);
    CKL();
    double normres0 = std::sqrt(host_sum_parts(D));
    const bool rc = recycling != 0 && (D.rc_cap > 0 || maxvec > 0);
    if (rc && D.rc_cap == 0) {  // the basis keeps the capacity of the first recycling solve
      D.rc_cap = maxvec;
      D.rcV = dalloc<double>((size_t)D.n * maxvec, own);
      D.rcW = dalloc<double>((size_t)D.n * maxvec, own);
      D.rc_part = dalloc<double>((size_t)D.npart * maxvec, own);
      D.rc_coef = dalloc<double>(maxvec, own);
      D.rc_nact_dev = dalloc<int>(1, own);
      CK(cudaMemsetAsync(D.rc_nact_dev, 0, sizeof(int), st));
      D.rc_nact = 0;
    }
    bool projected_done = false;
    if (rc && normres0 != 0.0 && D.rc_nact > 0) {
      // x += V V^T r, r -= S V V^T r (module_krylov.f90:373-452)
      k_rc_dots<<<D.npart, RT, 0, st>>>(D.n, D.rc_cap, D.rc_nact_dev, D.rcV, D.wsum, D.r, D.rc_part, nullptr);
      k_rc_coef<<<1, 256, 0, st>>>(D.rc_cap, D.rc_nact_dev, D.rc_part, D.npart, D.rc_coef, nullptr);
      CK(cudaMemsetAsync(D.z, 0, (size_t)D.n * sizeof(double), st));
      k_rc_combine<<<D.npart, RT, 0, st>>>(D.n, D.rc_nact_dev, D.rcV, D.rc_coef, 1.0, D.z, nullptr);
      CKL();
      k_axpy<<<(D.n + 255) / 256, 256, 0, st>>>(D.n, 1.0, D.z, D.x);
      CKL();
      launch_schur<T>(D, D.z, D.ap, true, nullptr, nullptr);
      k_axpy<<<(D.n + 255) / 256, 256, 0, st>>>(D.n, -1.0, D.ap, D.r);
      CKL();
      k_dot<<<D.npart, RT, 0, st>>>(D.n, D.r, D.r, D.wsum, D.part);
      CKL();
      if (std::sqrt(host_sum_parts(D)) / normres0 < tol) projected_done = true;  // no iteration needed
    }
    if (normres0 == 0.0 || projected_done) {
      postprocess = normres0 != 0.0;
    } else {
      launch_pc<T>(D, D.r, D.p, nullptr);
      double rmp = host_sum_parts(D);
      PcgCtl c{};
      c.rmp = rmp; c.normres0 = normres0; c.tol = tol; c.lastres = 1.0;
      c.iter = 1; c.maxit = maxit; c.ndecrmax = ndecrmax;
      CK(cudaMemcpyAsync(D.ctl, &c, sizeof(PcgCtl), cudaMemcpyHostToDevice, st));
      double tl = wall_time();
      D.prof.begin(PH_PCG, st);
      const int chunk = 4;
      int launched = 0;
      while (true) {
        for (int q = 0; q < chunk; ++q) {
          if (rc)  // S-orthogonalise p against the stored directions, twice (krylov_orthogonalize_icgs)
            for (int pass = 0; pass < 2; ++pass) {
              k_rc_dots<<<D.npart, RT, 0, st>>>(D.n, D.rc_cap, D.rc_nact_dev, D.rcW, D.wsum, D.p, D.rc_part, D.ctl);
              k_rc_coef<<<1, 256, 0, st>>>(D.rc_cap, D.rc_nact_dev, D.rc_part, D.npart, D.rc_coef, D.ctl);
              k_rc_combine<<<D.npart, RT, 0, st>>>(D.n, D.rc_nact_dev, D.rcV, D.rc_coef, -1.0, D.p, D.ctl);
              CKL();
            }
          launch_schur<T>(D, D.p, D.ap, false, D.ctl, D.p);
          k_sc_alpha<<<1, RT, 0, st>>>(D.ctl, D.part, D.npart);
          if (rc) {
            k_rc_store<<<D.npart, RT, 0, st>>>(D.n, D.rc_cap, D.rc_nact_dev, D.p, D.ap, D.rcV, D.rcW, D.ctl);
            k_rc_bump<<<1, 1, 0, st>>>(D.rc_cap, D.rc_nact_dev, D.ctl);
            CKL();
          }
          k_update_xr<<<D.npart, RT, 0, st>>>(D.n, D.ctl, D.x, D.r, D.p, D.ap, D.wsum, D.part);
          k_sc_res<<<1, RT, 0, st>>>(D.ctl, D.part, D.npart, D.hist);
          launch_pc<T>(D, D.r, D.z, D.ctl);
          k_sc_beta<<<1, RT, 0, st>>>(D.ctl, D.part, D.npart, D.diag, D.subdiag);
          k_update_p<<<D.npart, RT, 0, st>>>(D.n, D.ctl, D.p, D.z);
          CKL();
        }
        launched += chunk;
        CK(cudaMemcpyAsync(D.hctl, D.ctl, sizeof(PcgCtl), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (D.hctl->done || launched > maxit + chunk) break;
      }
      D.prof.end(PH_PCG, st);
      S.stats.t_iterations = wall_time() - tl;
      if (rc) {
        CK(cudaMemcpyAsync(&D.rc_nact, D.rc_nact_dev, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
      }
      PcgCtl c2 = *D.hctl;
      num_iter = c2.num_iter;
      reason = c2.reason;
      S.relres_history.resize(num_iter);
      if (num_iter > 0)
        CK(cudaMemcpyAsync(S.relres_history.data(), D.hist, num_iter * sizeof(double), cudaMemcpyDeviceToHost, st));
      int nw = c2.nw;
      vector<double> dg(std::max(nw, 1)), sd(std::max(nw, 1));
      if (nw > 1) {
        CK(cudaMemcpyAsync(dg.data(), D.diag, nw * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(sd.data(), D.subdiag, nw * sizeof(double), cudaMemcpyDeviceToHost, st));
      }
      CK(cudaStreamSynchronize(st));
      if (nw > 1) {
        sd.resize(nw - 1);
        cond = lanczos_max_eig(dg, sd);
      } else {
        cond = 1.0;
      }
    }
  }
  // interior values (module_levels.f90:4510-4576)
  double tp = wall_time();
  if (postprocess) {
    D.prof.begin(PH_POST, st);
    if (D.mixed)
      k_post_df<<<dim3((D.maxNO + POST_ROWS - 1) / POST_ROWS, D.nsub), 256, (D.maxNI + 1) * sizeof(float2), st>>>(
          D.ds, static_cast<const float*>(D.poolT), D.x, D.uniq, D.uo, D.uo_off);
    else
      k_post_f64<<<dim3((D.maxNO + 7) / 8, D.nsub), 256, 0, st>>>(D.ds, static_cast<const double*>(D.poolT), D.x,
                                                                  D.uniq, D.uo, D.uo_off);
    CKL();
    D.prof.end(PH_POST, st);
    // pull the solution into the subdomain arrays (dd_upload_solution semantics)
    vector<double> hx(D.n);
    size_t nuo = 0;
    for (auto& s : S.subs) nuo += s.ndofo;
    vector<double> huo(nuo);
    CK(cudaMemcpyAsync(hx.data(), D.x, D.n * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(huo.data(), D.uo, nuo * sizeof(double), cudaMemcpyDeviceToHost, st));
    g_d2h_bytes += (D.n + nuo) * sizeof(double);
    CK(cudaStreamSynchronize(st));
    for (int t = 0; t < D.nsub; ++t) {
      auto& s = S.subs[t];
      vector<double> u(s.ndof, 0.0);
      for (int q = 0; q < s.ndofo; ++q) u[s.iovsvn[s.operm[q]]] = huo[D.huo_off[t] + q];
      for (int i = 0; i < s.ndofi; ++i) u[s.iivsvn[i]] = hx[s.uniq[i]];
      s.sol = u;
    }
  }
  D.prof.end(PH_SOLVE_TOTAL, st);
  D.prof.collect();
  S.stats.h2d_bytes = g_h2d_bytes;
  S.stats.d2h_bytes = g_d2h_bytes;
  S.stats.t_postprocess = wall_time() - tp;
  S.stats.t_solve = wall_time() - t0;
  S.stats.num_iter = num_iter;
  S.stats.launches_solve = (double)(g_launches - launches0);
  if (stalled)
    throw Error{ERR_NUMERIC, "steepest descent: residual did not decrease for " + std::to_string(ndecrmax) +
                                 " iterations"};
  return true;
}

void device_set_profiling(Device* d, bool on) { d->prof.on = on; }

void device_get_profile(Device* d, double* ms, int* cnt) {
  d->prof.collect();
  for (int i = 0; i < NPHASE; ++i) { ms[i] = d->prof.ms[i]; cnt[i] = d->prof.cnt[i]; }
}

// New loads and boundary values after setup (module_levels.f90:855-903): the
// reduced-rhs inputs are uploaded again, v = A_oo^-1 f_o is recomputed with the
// existing factors (refined to FP64 accuracy in mixed mode) and written into
// the right-hand-side column of X, and g = f_i - A_io v is formed.  Factors,
// Schur complements and preconditioner stay as they are.
template <typename T>
static void ensure_nv(Device& D);
template <typename T>
static void reduced_rhs_device(Device& D);

template <typename T>
static void new_data_impl(Solver& S) {
  Device& D = *S.dev;
  const int nsub = D.nsub;
  cudaStream_t st = D.st;
  auto& own = D.owned;
  vector<long long> fooff(nsub), voff(nsub);
  long long nfo = 0, nv = 0;
  for (int t = 0; t < nsub; ++t) {
    fooff[t] = nfo; nfo += S.subs[t].ndofo;
    voff[t] = nv; nv += D.hs[t].NO;
  }
  vector<double> fov((size_t)std::max(1LL, nfo)), fir((size_t)std::max(1, D.nrep), 0.0);
#pragma omp parallel for schedule(dynamic)
  for (int t = 0; t < nsub; ++t) {
    vector<double> fo, fi;
    host_reduced_rhs_inputs(S.subs[t], fo, fi);
    std::copy(fo.begin(), fo.end(), fov.begin() + fooff[t]);
    std::copy(fi.begin(), fi.end(), fir.begin() + D.hs[t].rep);
  }
  CK(cudaMemcpyAsync(D.fo, fov.data(), nfo * sizeof(double), cudaMemcpyHostToDevice, st));
  CK(cudaMemcpyAsync(D.fi, fir.data(), D.nrep * sizeof(double), cudaMemcpyHostToDevice, st));
  g_h2d_bytes += (double)(nfo + D.nrep) * sizeof(double);
  (void)own; (void)nv; (void)voff;
  ensure_nv<T>(D);
  D.prof.begin(PH_NUMERIC_TOTAL, st, true);  // device part of setup_new_data
  reduced_rhs_device<T>(D);
  D.prof.end(PH_NUMERIC_TOTAL, st);
  int herr = 0;
  CK(cudaMemcpyAsync(&herr, D.err, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (herr) {
    CK(cudaMemsetAsync(D.err, 0, sizeof(int), st));  // reported once
    throw Error{ERR_NUMERIC, "device error flags " + std::to_string(herr) + " after new data"};
  }
}

// one-vector interior solve buffers (allocated on first use)
template <typename T>
static void ensure_nv(Device& D) {
  if (D.nv_v0) return;
  vector<long long> voff(D.nsub);
  long long nv = 0;
  for (int t = 0; t < D.nsub; ++t) { voff[t] = nv; nv += D.hs[t].NO; }
  D.nv_v0 = dalloc<T>(nv, D.owned);
  D.nv_v1 = dalloc<T>(nv, D.owned);
  D.nv_r = dalloc<T>(nv, D.owned);
  D.nv_off = upload(voff, D.owned, D.st);
}

// the reduced rhs of the current D.fo / D.fi on the device (module_dd.f90:6995-7257):
// the interior solve replaces the rhs column of X, grep = f_i - A_io X(:, ni)
template <typename T>
static void reduced_rhs_device(Device& D) {
  const int nsub = D.nsub;
  cudaStream_t st = D.st;
  T* v0 = static_cast<T*>(D.nv_v0);
  T* v1 = static_cast<T*>(D.nv_v1);
  T* rv = static_cast<T*>(D.nv_r);
  T* poolT = static_cast<T*>(D.poolT);
  const dim3 gv((D.maxNO + 127) / 128, nsub);
  const size_t smem = (size_t)(D.maxnbo * NB + 5 * NB) * sizeof(T);
  raise_smem(k_band_solve1<T>, smem);
  auto solve1 = [&](T* x) {
    k_band_solve1<T><<<nsub, NT, smem, st>>>(D.bd_oo, poolT, x, D.nv_off, D.bdu_oo);
    CKL();
  };
  k_fill_vec1<T><<<gv, 128, 0, st>>>(D.ds, D.fo, D.fo_off, v0, D.nv_off);
  CKL();
  solve1(v0);
  if constexpr (std::is_same_v<T, float>) {
    // two refinement steps with FP64-accurate residuals: v = v0 + (d1 + d2)
    k_residual1_df<<<gv, 128, 0, st>>>(D.ds, D.koo, D.fo, D.fo_off, v0, nullptr, v1, D.nv_off);
    CKL();
    solve1(v1);
    // as many further corrections as the setup's interior solves needed (at least one)
    for (int step = 2; step <= std::max(2, D.refine_steps); ++step) {
      k_residual1_df<<<gv, 128, 0, st>>>(D.ds, D.koo, D.fo, D.fo_off, v0, v1, rv, D.nv_off);
      CKL();
      solve1(rv);
      k_add_vec1<float><<<gv, 128, 0, st>>>(D.ds, rv, v1, D.nv_off);
      CKL();
    }
    k_put_rhs_column<float><<<gv, 128, 0, st>>>(D.ds, poolT, v0, v1, D.nv_off);
    CKL();
    k_reduced_rhs_df<<<dim3((D.maxNI + 127) / 128, nsub), 128, 0, st>>>(D.ds, D.kio, poolT, D.fi, D.grep);
    CKL();
  } else {
    k_put_rhs_column<double><<<gv, 128, 0, st>>>(D.ds, poolT, v0, nullptr, D.nv_off);
    CKL();
    k_reduced_rhs_f64<<<dim3((D.maxNI + 127) / 128, nsub), 128, 0, st>>>(D.ds, D.kio, poolT, D.fi, D.grep);
    CKL();
  }
}

// ------------------------------------------------------------ three levels
// The level-1 coarse problem is solved approximately by one BDDC application on
// level 2 (levels_corsub_standard_level + levels_solve_last_level +
// levels_add_standard_level, module_levels.f90:3849-4250): interior solves of
// the level-2 subdomains, the reduced rhs on the level-2 interface, the level-2
// BDDC preconditioner (with the exact level-3 coarse solve), interior resolve.
__global__ void k_l2_rhs(int nfo, const int* __restrict__ mo, int nrep, const int* __restrict__ mi,
                         const double* __restrict__ wi, const double* __restrict__ rc, double* __restrict__ fo,
                         double* __restrict__ fi) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < nfo) fo[g] = rc[mo[g]];
  if (g < nrep) fi[g] = mi[g] >= 0 ? wi[g] * rc[mi[g]] : 0.0;
}

__global__ void k_l2_out(int nfo, const int* __restrict__ mo, const double* __restrict__ uo, int nz,
                         const int* __restrict__ mz, const double* __restrict__ z, double* __restrict__ uc) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < nfo) uc[mo[g]] = uo[g];
  if (g < nz) uc[mz[g]] = z[g];
}

static void level2_apply(Device& D1, const double* rc, double* uc) {
  Solver& S2 = *D1.lev2;
  Device& D2 = *S2.dev;
  cudaStream_t st = D1.st;
  const int n1 = std::max(D2.l2_nfo, D2.nrep);
  k_l2_rhs<<<(n1 + 255) / 256, 256, 0, st>>>(D2.l2_nfo, D2.l2_mo, D2.nrep, D2.l2_mi, D2.l2_wi, rc, D2.fo, D2.fi);
  CKL();
  reduced_rhs_device<double>(D2);
  k_assemble_plain<<<(D2.n + 255) / 256, 256, 0, st>>>(D2.n, D2.own, D2.grep, nullptr, D2.g);
  CKL();
  launch_pc<double>(D2, D2.g, D2.z, nullptr);
  k_post_f64<<<dim3((D2.maxNO + 7) / 8, D2.nsub), 256, 0, st>>>(D2.ds, static_cast<const double*>(D2.poolT), D2.z,
                                                                 D2.uniq, D2.uo, D2.uo_off);
  CKL();
  const int n2 = std::max(D2.l2_nfo, D2.n);
  k_l2_out<<<(n2 + 255) / 256, 256, 0, st>>>(D2.l2_nfo, D2.l2_mo, D2.uo, D2.n, D2.l2_mz, D2.z, uc);
  CKL();
}

template <typename T>
static void setup_level2(Solver& S, Device& D) {
  cudaStream_t st = D.st;
  const int nsub = D.nsub;
  // local coarse matrices of the level-1 subdomains
  long long nsm = 0;
  for (auto& d : D.hs) nsm = std::max(nsm, d.oAc + (long long)d.ncp * d.ncp);
  vector<double> hsmall(std::max<long long>(1, nsm));
  CK(cudaMemcpyAsync(hsmall.data(), D.small, nsm * sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  vector<vector<double>> acs(nsub);
  if (D.mixed) {  // Phi^T S Phi with FP64-accurate products: the level-2 element matrices
    vector<int> all(nsub);
    std::iota(all.begin(), all.end(), 0);
    acs = coarse_energies<T>(D, all, nullptr);
  } else {
    for (int t = 0; t < nsub; ++t) {
      const DevSub& d = D.hs[t];
      acs[t].resize((size_t)d.nc * d.nc);
      for (int r = 0; r < d.nc; ++r)
        for (int c = 0; c < d.nc; ++c) acs[t][(size_t)r * d.nc + c] = hsmall[d.oAc + (long long)r * d.ncp + c];
    }
  }
  S.lev2 = host_build_level2(S, acs, S.prm.nsub2);
  Solver& S2 = *S.lev2;
  host_setup(S2);
  Error err{0, ""};
  S2.dev = device_create_on_stream(&D, err);
  if (!S2.dev) throw err;
  // the nested setup keeps this level's transfer and launch counters
  const double h2d = g_h2d_bytes, d2h = g_d2h_bytes;
  const long long nl = g_launches;
  const bool ok = device_setup(S2, err);
  g_h2d_bytes += h2d;
  g_d2h_bytes += d2h;
  g_launches += nl;
  if (!ok) throw err;
  Device& D2 = *S2.dev;
  ensure_nv<double>(D2);
  long long nfo = 0;
  for (auto& s2 : S2.subs) nfo += s2.ndofo;
  D2.l2_nfo = (int)nfo;
  vector<int> mo(std::max<long long>(1, nfo)), mi(std::max(1, D2.nrep), -1), mz(std::max(1, D2.n), 0);
  vector<double> wi(std::max(1, D2.nrep), 0.0);
  for (int t = 0; t < D2.nsub; ++t) {
    const Subdomain& q = S2.subs[t];
    const long long fo = D2.huo_off[t];
    for (int k = 0; k < q.ndofo; ++k) mo[fo + k] = q.isvgvn[q.iovsvn[q.operm[k]]];
    for (int i = 0; i < q.ndofi; ++i) {
      const int g = q.isvgvn[q.iivsvn[i]];
      mi[D2.hs[t].rep + i] = g;
      wi[D2.hs[t].rep + i] = q.wi[i];
      mz[q.uniq[i]] = g;
    }
  }
  // explicit interior inverses for the batched level-2 solves: A_oo X = I with the band factor
  {
    vector<BandDesc> bdi(D2.nsub);
    long long na = 0;
    int maxNO = 0;
    D2.l2_aoff.assign(D2.nsub, 0);
    for (int t = 0; t < D2.nsub; ++t) {
      const DevSub& d2 = D2.hs[t];
      D2.l2_aoff[t] = na;
      bdi[t] = D2.hbd_oo[t];
      bdi[t].ncol = d2.NO;
      bdi[t].oB = na;
      na += (long long)d2.NO * d2.NO;
      maxNO = std::max(maxNO, d2.NO);
    }
    D2.l2_ainv = dalloc<double>(std::max(1LL, na), D2.owned);
    CK(cudaMemsetAsync(D2.l2_ainv, 0, (size_t)std::max(1LL, na) * sizeof(double), st));
    const BandDesc* dbi = upload(bdi, D2.owned, st);
    k_band_identity<<<dim3((maxNO + 255) / 256, D2.nsub), 256, 0, st>>>(dbi, D2.l2_ainv);
    CKL();
    run_solve<double>(D2, dbi, D2.nsub, D2.maxnbo, maxNO, static_cast<const double*>(D2.poolT), D2.l2_ainv);
  }
  D2.l2_mo = upload(mo, D2.owned, st);
  D2.l2_mi = upload(mi, D2.owned, st);
  D2.l2_mz = upload(mz, D2.owned, st);
  D2.l2_wi = upload(wi, D2.owned, st);
  D.lev2 = &S2;
  CK(cudaStreamSynchronize(st));
}

}  // namespace bddc

#include "bddc_batch.cuh"

namespace bddc {

bool device_solve_batch(Solver& S, int nrhs, double tol, int maxit, int ndecrmax, vector<int>& num_iter,
                        vector<int>& reason, vector<double>& cond, Error& err) {
  try {
    if (S.dev->mixed) batch_solve_impl<float>(S, nrhs, tol, maxit, ndecrmax, num_iter, reason, cond);
    else batch_solve_impl<double>(S, nrhs, tol, maxit, ndecrmax, num_iter, reason, cond);
  } catch (Error& e) {
    err = e;
    return false;
  }
  return true;
}

bool device_new_data(Solver& S, Error& err) {
  try {
    if (!S.dev || !S.dev->ds) throw Error{ERR_ARGUMENT, "the preconditioner is not set up"};
    if (S.dev->mixed) new_data_impl<float>(S);
    else new_data_impl<double>(S);
  } catch (Error& e) {
    err = e;
    return false;
  }
  return true;
}

bool device_solve(Solver& S, int method, double tol, int maxit, int ndecrmax, int recycling, int maxvec,
                  int& num_iter, int& reason, double& cond, Error& err) {
  try {
    if (S.dev->mixed) return solve_impl<float>(S, method, tol, maxit, ndecrmax, recycling, maxvec, num_iter, reason, cond);
    return solve_impl<double>(S, method, tol, maxit, ndecrmax, recycling, maxvec, num_iter, reason, cond);
  } catch (Error& e) {
    err = e;
    return false;
  }
}

}  // namespace bddc
