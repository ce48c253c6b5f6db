// capi.cu -- extern "C" entry points of libpsfun_gb300 (see include/psfun_gb300.h).
#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"
#include "persist.cuh"

namespace psf {

static cudaStream_t g_stream = nullptr;
static bool g_stream_owned = false;
static thread_local std::string g_last_error;
static std::atomic<long long> g_launches{0};
static int g_sms = 0;

cudaStream_t stream() {
  if (!g_stream) {
    cudaStreamCreateWithFlags(&g_stream, cudaStreamNonBlocking);
    g_stream_owned = true;
  }
  return g_stream;
}
void set_last_error(const std::string& msg) { g_last_error = msg; }
void count_launch(int n) { g_launches += n; }
long long launch_count() { return g_launches.load(); }
int sm_count() {
  if (!g_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms <= 0) g_sms = 1;
  }
  return g_sms;
}

int DevBuf::ensure(size_t need) {
  if (need <= bytes && ptr) return PSFUN_SUCCESS;
  release();
  cudaError_t e = cudaMalloc(&ptr, need);
  if (e != cudaSuccess) {
    (void)cudaGetLastError();  // recoverable: keep it out of later launch checks
    ptr = nullptr;
    bytes = 0;
    set_last_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return PSFUN_ERR_ALLOC_DEALLOC;
  }
  bytes = need;
  return PSFUN_SUCCESS;
}
void DevBuf::release() {
  if (ptr) cudaFree(ptr);
  ptr = nullptr;
  bytes = 0;
}

// Fortran `character(len=20) :: s; s = val` then `select case (s)`.
void set_fstr(char* dst, const char* src) {
  size_t n = src ? strlen(src) : 0;
  if (n > 20) n = 20;
  memcpy(dst, src, n);
  dst[n] = 0;
}
bool fstr_eq(const char* s, const char* lit) {
  size_t ls = strlen(s), ll = strlen(lit);
  while (ls > 0 && s[ls - 1] == ' ') --ls;
  return ls == ll && strncmp(s, lit, ll) == 0;
}
static std::string upper_key(const char* what) {
  std::string k(what ? what : "");
  for (auto& ch : k) ch = (char)toupper((unsigned char)ch);
  while (!k.empty() && k.back() == ' ') k.pop_back();
  return k;
}

// ---- per-kernel timing ------------------------------------------------------
static bool g_prof = false;
struct ProfSlot {
  std::vector<cudaEvent_t> pool;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
  size_t next = 0;
  long long count = 0;
  double total_ms = 0.0;
};
static ProfSlot g_slots[PROF_N];
static cudaEvent_t prof_event(ProfSlot& sl) {
  if (sl.next == sl.pool.size()) {
    cudaEvent_t e;
    cudaEventCreate(&e);
    sl.pool.push_back(e);
  }
  return sl.pool[sl.next++];
}
bool prof_enabled() { return g_prof; }
void prof_begin(int k, cudaStream_t s) {
  if (!g_prof) return;
  ProfSlot& sl = g_slots[k];
  cudaEvent_t e = prof_event(sl);
  cudaEventRecord(e, s);
  sl.pending.push_back({e, nullptr});
}
void prof_end(int k, cudaStream_t s) {
  if (!g_prof) return;
  ProfSlot& sl = g_slots[k];
  cudaEvent_t e = prof_event(sl);
  cudaEventRecord(e, s);
  if (!sl.pending.empty()) sl.pending.back().second = e;
}
void prof_collect() {
  if (!g_prof) return;
  for (auto& sl : g_slots) {
    for (auto& pr : sl.pending) {
      float ms = 0.f;
      if (pr.second && cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess) {
        sl.total_ms += ms;
        sl.count += 1;
      }
    }
    sl.pending.clear();
    sl.next = 0;
  }
}

bool parse_fun(const psfun_serial* fun, FunParams* fp) {
  fp->scaling = fun->scaling;
  fp->padedegree = fun->padedegree;
  fp->phiorder = fun->phiorder;
  fp->fname = FN_INVALID;
  fp->variant = VAR_INVALID;
  if (fstr_eq(fun->fname, "EXP")) {
    fp->fname = FN_EXP;
    if (fstr_eq(fun->variant, "TAYLOR")) fp->variant = VAR_TAYLOR;
    else if (fstr_eq(fun->variant, "SASQ")) fp->variant = VAR_SASQ;
    else if (fstr_eq(fun->variant, "GENPADE")) fp->variant = VAR_GENPADE;
    else if (fstr_eq(fun->variant, "CHBHES")) fp->variant = VAR_CHBHES;
    else if (fstr_eq(fun->variant, "CHBGEN")) fp->variant = VAR_CHBGEN;
    else if (fstr_eq(fun->variant, "CHBSYM")) fp->variant = VAR_CHBSYM;
    else return false;  // includes the default 'EXPOKIT' (psfun_d_serial_mod.F90:387-390)
    if (fp->variant == VAR_GENPADE && (fun->padedegree < 1 || fun->padedegree > 60)) return false;
    return true;
  }
  if (fstr_eq(fun->fname, "PHI")) {
    fp->fname = FN_PHI;
    return fun->phiorder >= 1 && fun->padedegree >= 1 && fun->padedegree <= 60;
  }
  if (fstr_eq(fun->fname, "USERF")) {
    fp->fname = FN_USERF;
    if (fstr_eq(fun->variant, "SYM")) { fp->variant = VAR_SYM; return true; }
    return false;
  }
  return false;
}

// Self-test of the bounded device waits: a wait that nothing completes.
// which 0: a grid barrier of a 2-CTA cooperative grid whose target is one
// arrival more than the grid makes; which 1: an mbarrier wait for a phase
// that no thread or copy completes.  Both give up after kWaitLimitNs and
// record DEVERR_TIMEOUT, as every wait of the solvers does.
__global__ void k_selftest_wait(int which, unsigned* counter, int* err) {
  __shared__ uint64_t bar;
  if (which == 0) {
    if (grid_sync_to(counter, gridDim.x + 1u, err)) atomicOr(err, 0x100);  // completed: not expected
    return;
  }
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (mbar_wait(&bar, 0u)) atomicOr(err, 0x100);
    else atomicOr(err, DEVERR_TIMEOUT);
  }
}

}  // namespace psf

using namespace psf;

// ---------------------------------------------------------------------------
extern "C" {

int psfun_gpu_selftest_wait(int which) {
  if (which < 0 || which > 1) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  static DevBuf buf;
  PSF_TRY(buf.ensure(64));
  cudaStream_t s = stream();
  PSF_CUDA(cudaMemsetAsync(buf.ptr, 0, 64, s));
  unsigned* counter = buf.as<unsigned>();
  int* err = reinterpret_cast<int*>(counter + 4);
  if (which == 0) {
    void* args[] = {(void*)&which, (void*)&counter, (void*)&err};
    PSF_CUDA(cudaLaunchCooperativeKernel((void*)k_selftest_wait, dim3(2), dim3(32), args, 0, s));
  } else {
    k_selftest_wait<<<1, 32, 0, s>>>(which, counter, err);
  }
  count_launch();
  PSF_CUDA(cudaGetLastError());
  int h = 0;
  PSF_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  if (h & DEVERR_TIMEOUT) {
    set_last_error("self-test: the bounded device wait expired and reported it");
    return PSFUN_ERR_DEVICE_TIMEOUT;
  }
  set_last_error("self-test: the wait completed or reported nothing");
  return PSFUN_ERR_INTERNAL;
}

const char* psfun_gpu_version(void) { return "psfun_gb300 0.1 (sm_103a)"; }
const char* psfun_gpu_last_error(void) { return g_last_error.c_str(); }
long long psfun_gpu_kernel_launches(void) { return g_launches.load(); }

int psfun_gpu_set_stream(void* s) {
  if (g_stream && g_stream_owned) cudaStreamDestroy(g_stream);
  g_stream = (cudaStream_t)s;
  g_stream_owned = false;
  if (!s) stream();
  return PSFUN_SUCCESS;
}
void* psfun_gpu_get_stream(void) { return (void*)stream(); }

int psfun_gpu_profile_enable(int on) {
  g_prof = (on != 0);
  for (auto& sl : g_slots) {
    sl.count = 0;
    sl.total_ms = 0.0;
    sl.pending.clear();
    sl.next = 0;
  }
  return PSFUN_SUCCESS;
}

int psfun_gpu_profile_read(int kernel, long long* launches, double* total_ms) {
  if (kernel < 0 || kernel >= PROF_N) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  if (launches) *launches = g_slots[kernel].count;
  if (total_ms) *total_ms = g_slots[kernel].total_ms;
  return PSFUN_SUCCESS;
}

}  // extern "C"

// ---- CSR ------------------------------------------------------------------
// f(begin, end) over [0, n) in contiguous parts on up to 16 host threads
// (one part below 2^17 items).
template <class F>
static void host_parallel_for(int64_t n, F f) {
  const int T = std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
  if (n < ((int64_t)1 << 17) || T == 1) {
    f((int64_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(T);
  for (int t = 0; t < T; ++t) th.emplace_back([&, t] { f(n * t / T, n * (t + 1) / T); });
  for (auto& x : th) x.join();
}

extern "C" {

int psfun_gpu_csr_create(int64_t n, int64_t nnz, const int32_t* irp, const int32_t* ja, const double* val,
                         int index_base, psfun_csr** out) {
  if (!out) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  *out = nullptr;
  if (n < 0 || nnz < 0 || (n > 0 && !irp) || (nnz > 0 && (!ja || !val)) || (index_base != 0 && index_base != 1)) {
    set_last_error("invalid CSR arguments");
    return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  }
  if (n > 0x7ffffff0LL || nnz > 0x7ffffff0LL) {
    set_last_error("int32 CSR index overflow");
    return PSFUN_ERR_INVALID_MATRIX;
  }
  // validate + rebase to 0 (bit-exact: every index is checked, none is altered
  // other than the constant base shift)
  std::vector<int32_t> hirp(n + 1);
  if (n == 0) {
    hirp[0] = 0;
  } else {
    host_parallel_for(n + 1, [&](int64_t b, int64_t e) {
      for (int64_t i = b; i < e; ++i) hirp[i] = irp[i] - index_base;
    });
    if (hirp[0] != 0 || hirp[n] != nnz) {
      set_last_error("rowptr must start at the index base and end at nnz");
      return PSFUN_ERR_INVALID_MATRIX;
    }
    std::atomic<int> bad{0};
    host_parallel_for(n, [&](int64_t b, int64_t e) {
      for (int64_t i = b; i < e; ++i)
        if (hirp[i + 1] < hirp[i]) { bad.store(1); return; }
    });
    if (bad.load()) {
      set_last_error("rowptr not monotone");
      return PSFUN_ERR_INVALID_MATRIX;
    }
  }
  std::vector<int32_t> hja(nnz);
  {
    std::atomic<int> bad{0};
    host_parallel_for(nnz, [&](int64_t b, int64_t e) {
      for (int64_t k = b; k < e; ++k) {
        const int32_t c = ja[k] - index_base;
        if (c < 0 || c >= n) { bad.store(1); return; }
        hja[k] = c;
      }
    });
    if (bad.load()) {
      set_last_error("column index out of range");
      return PSFUN_ERR_INVALID_MATRIX;
    }
  }
  auto* a = new psfun_csr();
  a->n = n;
  a->nnz = nnz;
  // tile schedule
  std::vector<int32_t> tiles;
  tiles.reserve(n / kTileRows + 16);
  int64_t r = 0;
  while (r < n) {
    tiles.push_back((int32_t)r);
    const int64_t start = r;
    int64_t acc = 0;
    while (r < n && r - start < kTileRows && acc + (hirp[r + 1] - hirp[r]) <= kTileNnz) {
      acc += hirp[r + 1] - hirp[r];
      ++r;
    }
    if (r == start) ++r;  // a row longer than a tile: its own tile
  }
  tiles.push_back((int32_t)n);
  a->ntiles = (int32_t)tiles.size() - 1;
  std::vector<int2> tdesc(tiles.size());
  for (size_t t = 0; t < tiles.size(); ++t) {
    tdesc[t].x = tiles[t];
    tdesc[t].y = hirp[tiles[t]];
    if (t + 1 < tiles.size()) a->max_tile_rows = std::max<int32_t>(a->max_tile_rows, tiles[t + 1] - tiles[t]);
  }
  // norms and diagonal (per row; the maxima combined over the parts)
  a->h_diag.assign(n, 0.0);
  std::mutex mx;
  double ninf = 0.0;
  int32_t max_row = 0;
  host_parallel_for(n, [&](int64_t b, int64_t e) {
    double ninf_p = 0.0;
    int32_t max_row_p = 0;
    for (int64_t i = b; i < e; ++i) {
      double s = 0.0;
      max_row_p = std::max<int32_t>(max_row_p, hirp[i + 1] - hirp[i]);
      for (int32_t k = hirp[i]; k < hirp[i + 1]; ++k) {
        s += fabs(val[k]);
        if (hja[k] == i) a->h_diag[i] += val[k];
      }
      if (s > ninf_p) ninf_p = s;
    }
    std::lock_guard<std::mutex> lock(mx);
    ninf = std::max(ninf, ninf_p);
    max_row = std::max(max_row, max_row_p);
  });
  a->norm_inf = ninf;
  a->max_row = max_row;
  cudaStream_t s = stream();
  auto fail = [&](cudaError_t e) {
    (void)cudaGetLastError();
    set_last_error(std::string("csr_create: ") + cudaGetErrorString(e));
    psfun_gpu_csr_destroy(a);
    return PSFUN_ERR_CUDA;
  };
  cudaError_t e;
  // padded allocations so that 16-byte bulk copies never leave the buffers
  if ((e = cudaMalloc(&a->irp, sizeof(int32_t) * (n + 1 + 8))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&a->ja, sizeof(int32_t) * (nnz + 16))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&a->val, sizeof(double) * (nnz + 8))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&a->tile_row, sizeof(int32_t) * tiles.size())) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&a->sched, 4 * sizeof(unsigned))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&a->tile_desc, sizeof(int2) * tdesc.size())) != cudaSuccess) return fail(e);
  if ((e = cudaMemcpyAsync(a->tile_desc, tdesc.data(), sizeof(int2) * tdesc.size(), cudaMemcpyHostToDevice, s)) !=
      cudaSuccess)
    return fail(e);
  cudaMemsetAsync(a->sched, 0, 4 * sizeof(unsigned), s);
  cudaMemsetAsync(a->ja, 0, sizeof(int32_t) * (nnz + 16), s);
  cudaMemsetAsync(a->val, 0, sizeof(double) * (nnz + 8), s);
  if ((e = cudaMemcpyAsync(a->irp, hirp.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return fail(e);
  if (nnz > 0) {
    if ((e = cudaMemcpyAsync(a->ja, hja.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return fail(e);
    if ((e = cudaMemcpyAsync(a->val, val, sizeof(double) * nnz, cudaMemcpyHostToDevice, s)) != cudaSuccess)
      return fail(e);
  }
  if ((e = cudaMemcpyAsync(a->tile_row, tiles.data(), sizeof(int32_t) * tiles.size(), cudaMemcpyHostToDevice, s)) !=
      cudaSuccess)
    return fail(e);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(e);
  *out = a;
  return PSFUN_SUCCESS;
}

int psfun_gpu_csr_destroy(psfun_csr* a) {
  if (!a) return PSFUN_SUCCESS;
  if (a->T) psfun_gpu_csr_destroy(a->T);
  if (a->bj_val) cudaFree(a->bj_val);
  if (a->bj_col) cudaFree(a->bj_col);
  if (a->bj_rowoff) cudaFree(a->bj_rowoff);
  if (a->bj_cnt) cudaFree(a->bj_cnt);
  if (a->bj_udinv) cudaFree(a->bj_udinv);
  if (a->irp) cudaFree(a->irp);
  if (a->ja) cudaFree(a->ja);
  if (a->val) cudaFree(a->val);
  if (a->tile_row) cudaFree(a->tile_row);
  if (a->diag_inv) cudaFree(a->diag_inv);
  if (a->sched) cudaFree(a->sched);
  if (a->tile_desc) cudaFree(a->tile_desc);
  delete a;
  return PSFUN_SUCCESS;
}

int psfun_gpu_csr_info(const psfun_csr* a, int64_t* n, int64_t* nnz, int64_t* ntiles, double* norm_inf) {
  if (!a) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  if (n) *n = a->n;
  if (nnz) *nnz = a->nnz;
  if (ntiles) *ntiles = a->ntiles;
  if (norm_inf) *norm_inf = a->norm_inf;
  return PSFUN_SUCCESS;
}

int psfun_gpu_csr_is_symmetric(psfun_csr* a, int* sym) {
  psf::NvtxRange nvtx_range("psfun_gpu_csr_is_symmetric");
  if (!a || !sym) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  return psf::csr_symmetric(a, sym);
}

}  // extern "C"

namespace psf {

int csr_download(psfun_csr* a, std::vector<int32_t>& irp, std::vector<int32_t>& ja, std::vector<double>& val) {
  irp.resize(a->n + 1);
  ja.resize(a->nnz);
  val.resize(a->nnz);
  cudaStream_t s = stream();
  PSF_CUDA(cudaMemcpyAsync(irp.data(), a->irp, sizeof(int32_t) * (a->n + 1), cudaMemcpyDeviceToHost, s));
  if (a->nnz > 0) {
    PSF_CUDA(cudaMemcpyAsync(ja.data(), a->ja, sizeof(int32_t) * a->nnz, cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaMemcpyAsync(val.data(), a->val, sizeof(double) * a->nnz, cudaMemcpyDeviceToHost, s));
  }
  PSF_CUDA(cudaStreamSynchronize(s));
  return PSFUN_SUCCESS;
}

// Transpose by a counting sort over the columns: traversing the rows in
// order leaves every row of the transpose in increasing column order.
static void host_transpose(int64_t n, const std::vector<int32_t>& irp, const std::vector<int32_t>& ja,
                           const std::vector<double>& val, std::vector<int32_t>& irpT, std::vector<int32_t>& jaT,
                           std::vector<double>& valT) {
  const int64_t nnz = (int64_t)ja.size();
  irpT.assign(n + 1, 0);
  for (int64_t k = 0; k < nnz; ++k) ++irpT[ja[k] + 1];
  for (int64_t i = 0; i < n; ++i) irpT[i + 1] += irpT[i];
  std::vector<int32_t> cur(irpT.begin(), irpT.end() - 1);
  jaT.resize(nnz);
  valT.resize(nnz);
  for (int64_t i = 0; i < n; ++i)
    for (int32_t k = irp[i]; k < irp[i + 1]; ++k) {
      const int32_t pos = cur[ja[k]]++;
      jaT[pos] = (int32_t)i;
      valT[pos] = val[k];
    }
}

int csr_symmetric(psfun_csr* a, int* sym) {
  if (a->sym >= 0) {
    *sym = a->sym;
    return PSFUN_SUCCESS;
  }
  std::vector<int32_t> irp, ja, irpT, jaT;
  std::vector<double> val, valT;
  PSF_TRY(csr_download(a, irp, ja, val));
  host_transpose(a->n, irp, ja, val, irpT, jaT, valT);
  int ok = (irp == irpT) ? 1 : 0;
  std::vector<std::pair<int32_t, double>> ra, rt;
  for (int64_t i = 0; ok && i < a->n; ++i) {
    const int32_t b = irp[i], e = irp[i + 1];
    bool sorted = true;
    for (int32_t k = b + 1; k < e; ++k)
      if (ja[k] <= ja[k - 1]) { sorted = false; break; }
    if (sorted) {
      for (int32_t k = b; k < e && ok; ++k)
        if (ja[k] != jaT[k] || !(val[k] == valT[k])) ok = 0;
    } else {  // unsorted row or repeated entries: compare as sorted (column, value) lists
      ra.clear();
      rt.clear();
      for (int32_t k = b; k < e; ++k) {
        ra.emplace_back(ja[k], val[k]);
        rt.emplace_back(jaT[k], valT[k]);
      }
      std::sort(ra.begin(), ra.end());
      std::sort(rt.begin(), rt.end());
      for (size_t q = 0; q < ra.size() && ok; ++q)
        if (ra[q].first != rt[q].first || !(ra[q].second == rt[q].second)) ok = 0;
    }
  }
  a->sym = ok;
  *sym = ok;
  return PSFUN_SUCCESS;
}

int csr_transpose(psfun_csr* a, psfun_csr** out) {
  if (!a->T) {
    std::vector<int32_t> irp, ja, irpT, jaT;
    std::vector<double> val, valT;
    PSF_TRY(csr_download(a, irp, ja, val));
    host_transpose(a->n, irp, ja, val, irpT, jaT, valT);
    psfun_csr* t = nullptr;
    PSF_TRY(psfun_gpu_csr_create(a->n, a->nnz, irpT.data(), jaT.data(), valT.data(), 0, &t));
    a->T = t;
  }
  *out = a->T;
  return PSFUN_SUCCESS;
}

// y = alpha A x + beta y through the warp-specialised tile pipeline of the
// persistent kernels (persist.cuh): one block per SM over a contiguous range
// of tiles, the last warp staging up to four tiles ahead by TMA.
__global__ void __launch_bounds__(kSpmvThreads) k_spmv_axpby(CsrDev A, const double* x, double alpha, double beta,
                                                             double* y, int* err, int tiles_per_cta) {
  extern __shared__ __align__(128) unsigned char lz_smem_raw[];
  LzSmem& sm = *reinterpret_cast<LzSmem*>(lz_smem_raw);
  const int t0 = min(A.ntiles, (int)blockIdx.x * tiles_per_cta);
  const int t1 = min(A.ntiles, t0 + tiles_per_cta);
  if (t0 >= t1) return;
  lz_smem_init(sm);
  const bool stream = A.stream != 0;
  PipeCounters pc{0u, 0u};
  if (threadIdx.x == kConsumerWarps * 32) {
    if (!pipe_produce(A, t0, t0 + min(kLzStages, t1 - t0), sm, pc.issued, stream)) atomicOr(err, DEVERR_TIMEOUT);
  }
  EpiAxpby epi{alpha, beta, y};
  pipe_spmv(A, x, t0, t1, sm, epi, err, pc, false, stream);
}

int spmv_device(psfun_csr* a, double alpha, const double* x, double beta, double* y) {
  static DevBuf errbuf;
  PSF_TRY(errbuf.ensure(sizeof(int)));
  cudaStream_t s = stream();
  PSF_CUDA(cudaMemsetAsync(errbuf.ptr, 0, sizeof(int), s));
  if (a->ntiles > 0) {
    static const int gmax = persist_grid_for(k_spmv_axpby);
    const int tpc = std::max(1, (a->ntiles + gmax - 1) / gmax);
    const int g = std::max(1, (a->ntiles + tpc - 1) / tpc);
    k_spmv_axpby<<<g, kSpmvThreads, kLzSmemBytes, s>>>(a->dev(), x, alpha, beta, y, errbuf.as<int>(), tpc);
    count_launch();
    PSF_CUDA(cudaGetLastError());
  }
  int herr = 0;
  PSF_CUDA(cudaMemcpyAsync(&herr, errbuf.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  if (herr & DEVERR_TIMEOUT) return PSFUN_ERR_DEVICE_TIMEOUT;
  return PSFUN_SUCCESS;
}
}  // namespace psf

extern "C" {

int psfun_gpu_csr_spmv_device(psfun_csr* a, double alpha, const double* x, double beta, double* y) {
  psf::NvtxRange nvtx_range("psfun_gpu_csr_spmv_device");
  if (!a || !x || !y) return PSFUN_ERR_INVALID_VECT_STATE;
  return spmv_device(a, alpha, x, beta, y);
}

int psfun_gpu_csr_spmv(psfun_csr* a, double alpha, const double* x, double beta, double* y) {
  psf::NvtxRange nvtx_range("psfun_gpu_csr_spmv");
  if (!a || !x || !y) return PSFUN_ERR_INVALID_VECT_STATE;
  const size_t nb = sizeof(double) * (a->n + 1);
  DevBuf dx, dy;
  PSF_TRY(dx.ensure(nb));
  if (dy.ensure(nb) != PSFUN_SUCCESS) { dx.release(); return PSFUN_ERR_ALLOC_DEALLOC; }
  cudaStream_t s = stream();
  int rc = PSFUN_SUCCESS;
  if (cudaMemcpyAsync(dx.ptr, x, sizeof(double) * a->n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(dy.ptr, y, sizeof(double) * a->n, cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = PSFUN_ERR_CUDA;
  if (rc == PSFUN_SUCCESS) rc = spmv_device(a, alpha, dx.as<double>(), beta, dy.as<double>());
  if (rc == PSFUN_SUCCESS) {
    if (cudaMemcpyAsync(y, dy.ptr, sizeof(double) * a->n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      rc = PSFUN_ERR_CUDA;
  }
  dx.release();
  dy.release();
  return rc;
}

// ---- serial function object -------------------------------------------------
int psfun_gpu_serial_create(psfun_serial** out) {
  if (!out) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  auto* f = new psfun_serial();
  set_fstr(f->fname, "EXP");
  set_fstr(f->variant, "EXPOKIT");
  *out = f;
  return PSFUN_SUCCESS;
}
int psfun_gpu_serial_destroy(psfun_serial* fun) {
  delete fun;
  return PSFUN_SUCCESS;
}
int psfun_gpu_serial_set_string(psfun_serial* fun, const char* what, const char* val) {
  if (!fun || !val) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  const std::string k = upper_key(what);
  if (k == "FNAME") set_fstr(fun->fname, val);
  else if (k == "VARIANT") set_fstr(fun->variant, val);
  else return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  return PSFUN_SUCCESS;
}
int psfun_gpu_serial_set_real(psfun_serial* fun, const char* what, double val) {
  if (!fun) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  if (upper_key(what) == "SCALING") { fun->scaling = val; return PSFUN_SUCCESS; }
  return PSFUN_ERR_INVALID_ARGS_COMBINATION;
}
int psfun_gpu_serial_set_integer(psfun_serial* fun, const char* what, int val) {
  if (!fun) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  const std::string k = upper_key(what);
  if (k == "PADE_DEGREE") fun->padedegree = val;
  else if (k == "PHIORDER") fun->phiorder = val;
  else return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  return PSFUN_SUCCESS;
}
int psfun_gpu_serial_set_function(psfun_serial* fun, const char* what, psfun_userf val) {
  if (!fun) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  if (upper_key(what) == "FPOINTER") { fun->f_ptr = val; return PSFUN_SUCCESS; }
  return PSFUN_ERR_INVALID_ARGS_COMBINATION;
}
int psfun_gpu_serial_get(const psfun_serial* fun, char* fname, char* variant, double* scaling, int* padedegree,
                         int* phiorder) {
  if (!fun) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  if (fname) strcpy(fname, fun->fname);
  if (variant) strcpy(variant, fun->variant);
  if (scaling) *scaling = fun->scaling;
  if (padedegree) *padedegree = fun->padedegree;
  if (phiorder) *phiorder = fun->phiorder;
  return PSFUN_SUCCESS;
}

int psfun_gpu_serial_apply(psfun_serial* fun, int n, const double* a, int lda, double* y, const double* x) {
  psf::NvtxRange nvtx_range("psfun_gpu_serial_apply");
  if (!fun || !a || !x || !y) return PSFUN_ERR_INVALID_VECT_STATE;
  if (n < 1 || lda < n) return PSFUN_ERR_FROM_SUBROUTINE;
  static DevBuf da, dx, dy;  // kept between calls, grown as needed
  PSF_TRY(da.ensure(sizeof(double) * (size_t)n * n));
  PSF_TRY(dx.ensure(sizeof(double) * n));
  PSF_TRY(dy.ensure(sizeof(double) * n));
  cudaStream_t s = stream();
  int rc = PSFUN_SUCCESS;
  if (cudaMemcpy2DAsync(da.ptr, sizeof(double) * n, a, sizeof(double) * lda, sizeof(double) * n, n,
                        cudaMemcpyHostToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(dx.ptr, x, sizeof(double) * n, cudaMemcpyHostToDevice, s) != cudaSuccess)
    rc = PSFUN_ERR_CUDA;
  if (rc == PSFUN_SUCCESS) rc = serial_apply_device(fun, n, da.as<double>(), n, dy.as<double>(), dx.as<double>());
  if (rc == PSFUN_SUCCESS) {
    if (cudaMemcpyAsync(y, dy.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      rc = PSFUN_ERR_CUDA;
  }
  return rc;
}

}  // extern "C"

namespace psf {
// COO -> dense n x n on the device (psfun_d_serial_apply_sparse, :547-559)
__global__ void k_csr_to_dense(CsrDev A, double* D) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < A.n; r += (int64_t)gridDim.x * blockDim.x)
    for (int32_t k = A.irp[r]; k < A.irp[r + 1]; ++k) D[r + (size_t)A.ja[k] * A.n] = A.val[k];
}
}  // namespace psf

extern "C" {

int psfun_gpu_serial_apply_sparse(psfun_serial* fun, psfun_csr* a, double* y, const double* x) {
  psf::NvtxRange nvtx_range("psfun_gpu_serial_apply_sparse");
  if (!fun || !a || !x || !y) return PSFUN_ERR_INVALID_VECT_STATE;
  const int64_t n = a->n;
  if (n < 1 || n > 8192) return PSFUN_ERR_FROM_SUBROUTINE;
  static DevBuf da, dx, dy;  // kept between calls, grown as needed
  PSF_TRY(da.ensure(sizeof(double) * (size_t)n * n));
  PSF_TRY(dx.ensure(sizeof(double) * n));
  PSF_TRY(dy.ensure(sizeof(double) * n));
  cudaStream_t s = stream();
  int rc = PSFUN_SUCCESS;
  cudaMemsetAsync(da.ptr, 0, sizeof(double) * (size_t)n * n, s);
  k_csr_to_dense<<<(int)((n + 255) / 256), 256, 0, s>>>(a->dev(), da.as<double>());
  count_launch();
  if (cudaMemcpyAsync(dx.ptr, x, sizeof(double) * n, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = PSFUN_ERR_CUDA;
  if (rc == PSFUN_SUCCESS) rc = serial_apply_device(fun, (int)n, da.as<double>(), (int)n, dy.as<double>(), dx.as<double>());
  if (rc == PSFUN_SUCCESS) {
    if (cudaMemcpyAsync(y, dy.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      rc = PSFUN_ERR_CUDA;
  }
  return rc;
}

// ---- Krylov method object ------------------------------------------------------
int psfun_gpu_krylov_create(psfun_krylov** out) {
  if (!out) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  auto* m = new psfun_krylov();
  set_fstr(m->kname, "ARNOLDI");
  set_fstr(m->kmethd, "CG");
  *out = m;
  return PSFUN_SUCCESS;
}
int psfun_gpu_krylov_destroy(psfun_krylov* meth) {
  if (!meth) return PSFUN_SUCCESS;
  meth->V.release();
  meth->u.release();
  meth->small.release();
  meth->scratch.release();
  meth->partials.release();
  meth->dgroup.release();
  meth->ctrl.release();
  meth->xy.release();
  if (meth->graph) cudaGraphExecDestroy(meth->graph);
  delete meth;
  return PSFUN_SUCCESS;
}
int psfun_gpu_krylov_set_string(psfun_krylov* meth, const char* what, const char* val) {
  if (!meth || !val) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  const std::string k = upper_key(what);
  if (k == "KNAME") { set_fstr(meth->kname, val); return PSFUN_SUCCESS; }
  if (k == "KMETHD") { set_fstr(meth->kmethd, val); return PSFUN_SUCCESS; }
  if (k == "PREC") {
    const std::string v = upper_key(val);
    if (v == "NONE" || v == "NOPREC") meth->prec = 0;
    else if (v == "DIAG") meth->prec = 1;
    else if (v == "BJAC") meth->prec = 2;
    else return PSFUN_ERR_INVALID_ARGS_COMBINATION;
    return PSFUN_SUCCESS;
  }
  return PSFUN_ERR_INVALID_ARGS_COMBINATION;
}
int psfun_gpu_krylov_precinit(psfun_krylov* meth, const char* ptype) {
  if (!meth || !ptype) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  const std::string v = upper_key(ptype);
  if (v == "NONE" || v == "NOPREC") meth->prec = 0;
  else if (v == "DIAG") meth->prec = 1;
  else if (v == "BJAC") meth->prec = 2;
  else {
    psf::set_last_error("precinit: preconditioner type '" + v +
                        "' is not available (NOPREC, NONE, DIAG and BJAC are)");
    return PSFUN_ERR_FROM_SUBROUTINE;
  }
  return PSFUN_SUCCESS;
}
int psfun_gpu_krylov_precbuild(psfun_krylov* meth, psfun_csr* a) {
  psf::NvtxRange nvtx_range("psfun_gpu_krylov_precbuild");
  if (!meth || !a) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  if (meth->prec == 1) PSF_TRY(psf::csr_build_diag_inv(a));
  if (meth->prec == 2) PSF_TRY(psf::csr_build_bjac(a));
  return PSFUN_SUCCESS;
}
int psfun_gpu_krylov_set_real(psfun_krylov* meth, const char* what, double val) {
  if (!meth) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  const std::string k = upper_key(what);
  if (k == "TAU") { meth->tau = val; return PSFUN_SUCCESS; }
  return PSFUN_ERR_INVALID_ARGS_COMBINATION;
}
int psfun_gpu_krylov_set_integer(psfun_krylov* meth, const char* what, int val) {
  if (!meth) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  const std::string k = upper_key(what);
  if (k == "ITMAX") meth->itmax = val;
  else if (k == "ITRACE") meth->itrace = val;
  else if (k == "ISTOPC") meth->istopc = val;
  else if (k == "IRST") meth->irst = val;
  else if (k == "KEEPLAST") meth->keeplast = val;
  else if (k == "BATCHMAP" && val >= -1 && val <= 2) meth->batchmap = val;
  else return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  return PSFUN_SUCCESS;
}

int psfun_gpu_d_krylov_apply_device(psfun_krylov* meth, psfun_serial* fun, psfun_csr* a, double* y,
                                    const double* x, double eps, int itmax, int itrace, int istop, int* iter,
                                    double* err, double* res, int res_cap, int* res_len) {
  psf::NvtxRange nvtx_range("psfun_gpu_d_krylov_apply_device");
  if (!meth || !fun || !a) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  return krylov_apply_device(meth, fun, a, y, x, eps, itmax, itrace, istop, iter, err, res, res_cap, res_len);
}

// The device address of host memory that is pinned and mapped into the
// device's address space (cudaHostAlloc, cudaHostRegister), else null:
// pageable memory is staged through device buffers instead.
static void* mapped_device_ptr(const void* p) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return nullptr;
  }
  if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
  return at.devicePointer;
}

int psfun_gpu_d_krylov_apply(psfun_krylov* meth, psfun_serial* fun, psfun_csr* a, double* y, const double* x,
                             double eps, int itmax, int itrace, int istop, int* iter, double* err, double* res,
                             int res_cap, int* res_len) {
  psf::NvtxRange nvtx_range("psfun_gpu_d_krylov_apply");
  if (!meth || !fun || !a) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  if (!x || !y) return PSFUN_ERR_INVALID_VECT_STATE;
  const int64_t n = a->n;
  const size_t vb = sizeof(double) * (size_t)((n + 31) & ~31LL);
  PSF_TRY(meth->xy.ensure(2 * vb + 64));
  double* dx = meth->xy.as<double>();
  double* dy = reinterpret_cast<double*>(meth->xy.as<char>() + vb);
  cudaStream_t s = stream();
  // Pinned, mapped host vectors are read and written by the kernels in place
  // (x once by the first kernel, y once by the assembly), over the
  // CPU-GPU link, instead of through staging copies; x is staged when it
  // shares memory with y.
  const double* mx = static_cast<const double*>(mapped_device_ptr(x));
  double* my = static_cast<double*>(mapped_device_ptr(y));
  if (mx && my) {
    const char *xb = reinterpret_cast<const char*>(x), *yb = reinterpret_cast<const char*>(y);
    const size_t len = sizeof(double) * (size_t)n;
    if (xb < yb + len && yb < xb + len) mx = nullptr;
  }
  if (mx) dx = const_cast<double*>(mx);
  else PSF_CUDA(cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  if (my) dy = my;
  const int rc = krylov_apply_device(meth, fun, a, dy, dx, eps, itmax, itrace, istop, iter, err, res, res_cap, res_len);
  if (rc != PSFUN_SUCCESS) return rc;
  if (!my) PSF_CUDA(cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  return PSFUN_SUCCESS;
}

}  // extern "C"
