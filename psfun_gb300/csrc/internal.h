// internal.h -- host-side handle types and helpers of libpsfun_gb300.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/psfun_gb300.h"
#include <nvtx3/nvToolsExt.h>
#include "dense.cuh"
#include "spmv.cuh"

namespace psf {

// Library-wide state.
cudaStream_t stream();
void set_last_error(const std::string& msg);
void count_launch(int n = 1);
long long launch_count();
int sm_count();

// CUDA call -> status code, recording the message.  A failed call's error is
// also taken off the runtime's last-error slot (cudaGetLastError), so that a
// recoverable failure (an allocation the device cannot satisfy) is not
// reported again by the next call's launch checks.
#define PSF_CUDA(call)                                                          \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      (void)cudaGetLastError();                                                 \
      ::psf::set_last_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
      return PSFUN_ERR_CUDA;                                                    \
    }                                                                           \
  } while (0)

#define PSF_TRY(expr)        \
  do {                               \
    int rc_ = (expr);                \
    if (rc_ != PSFUN_SUCCESS) return rc_; \
  } while (0)

// Device buffer that grows on demand (never shrinks until freed).
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
  int ensure(size_t need);
  void release();
  template <class T>
  T* as() const { return static_cast<T*>(ptr); }
};

// An NVTX range over one C-ABI call (named after the entry point), for
// profilers; without a tool attached it costs a null check.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// Control block of one Krylov solve, in device memory.
struct KCtrl {
  int done;       // stop enqueued work
  int conv;       // estimate below eps
  int breakdown;  // Lanczos |beta| < 1e-16 / Arnoldi h(i,i-1) == 0
  int itx;        // iterations (reference `itx`)
  int yk_len;
  int nterms;
  int err;        // DEVERR_* flags
  int info;       // PSBLAS-style status
  unsigned bar_count;
  unsigned bar_gen;
  unsigned red_counter;
  unsigned red_counter2;
  // monitor CTA of a persistent Lanczos launch (shifted residuals or the
  // a posteriori estimate running beside the steps); on a cache line of
  // their own, away from the grid barrier's counter that the monitor's
  // polling would otherwise slow down
  alignas(128) int pub;  // last Lanczos step whose T entries are published (CTA 0)
  int stop_req;   // the monitor asks the steps to stop
  int stop_dec;   // CTA 0's reading of stop_req, taken before a grid barrier
  int bd_step;    // step at which a Lanczos breakdown was found (0: none)
  int conv_first; // concurrent estimates: the first converged iteration (INT_MAX: none)
  int est_last;   // concurrent estimates: the last iteration estimated
  int steps_end;  // persistent Arnoldi: 1 + the last step published, once the steps have ended (0: running)
  alignas(128) double beta0;  // rs(1) = ||x||
  double errnum;
  double errden;
  double c1, c2;  // Lanczos update coefficients
  double derr;
};

}  // namespace psf

struct psfun_csr {
  int64_t n = 0, nnz = 0;
  int32_t* irp = nullptr;
  int32_t* ja = nullptr;
  double* val = nullptr;
  int32_t* tile_row = nullptr;
  int32_t ntiles = 0;
  double norm_inf = 0.0;
  double* diag_inv = nullptr;  // Jacobi preconditioner (lazy)
  unsigned* sched = nullptr;   // SpMV tile work counter + blocks-done counter (zero between launches)
  int2* tile_desc = nullptr;   // per tile {first row, first stored entry}, ntiles + 1 entries
  int32_t max_tile_rows = 0;
  int32_t max_row = 0;         // longest row (stored entries)
  std::vector<double> h_diag;  // diagonal of A (host copy, for DIAG)
  // BJAC preconditioner (lazy): ILU(0) factors of the diagonal blocks of
  // kBjacRows consecutive rows, laid out for a warp that solves 32 blocks at
  // once (lane = block): for block group g (blocks 32 g .. 32 g + 31) and row
  // r of the blocks, the row's L then U entries as slots of 32 lanes
  // (bj_val: value, bj_col: column within the block; zero padding to the
  // group's longest row), bj_rowoff[32 g + r] the first slot, bj_cnt[32 g + r]
  // the L and U slot counts, bj_udinv[(32 g + r) * 32 + lane] the reciprocal
  // pivot.
  double* bj_val = nullptr;
  uint8_t* bj_col = nullptr;
  int32_t* bj_rowoff = nullptr;
  uchar2* bj_cnt = nullptr;
  double* bj_udinv = nullptr;
  int sym = -1;                // A == A^T (pattern and values): 1 yes, 0 no, -1 not yet checked
  psfun_csr* T = nullptr;      // A^T as its own handle, built on first use (nonsymmetric A)
  psf::CsrDev dev() const {
    psf::CsrDev d;
    d.n = n; d.nnz = nnz; d.irp = irp; d.ja = ja; d.val = val; d.tile_row = tile_row; d.ntiles = ntiles;
    d.sched = sched;
    d.tile_desc = tile_desc;
    d.stream = (nnz * 12 + n * 4) > ((int64_t)64 << 20) ? 1 : 0;
    return d;
  }
};

struct psfun_serial {
  char fname[21];
  char variant[21];
  double scaling = 1.0;
  int padedegree = 6;
  int phiorder = 1;
  psfun_userf f_ptr = nullptr;
};

struct psfun_krylov {
  char kname[21];
  char kmethd[21];
  double tau = 0.0;
  int itmax = 200, itrace = 0, istopc = 1, irst = 10;
  int keeplast = 0;
  int batchmap = -1;  // SpMM mapping of the batched Lanczos: -1 chosen by the autotuner, 0..2 fixed
  int prec = 0;  // inner-solve preconditioner of SAIARNOLDI: 0 NONE, 1 DIAG
  // cached workspace (never per call)
  psf::DevBuf V, u, small, scratch, partials, ctrl, xy;
  psf::DevBuf dgroup;  // DenseGroup of the dense f(H) kernels
  psf::DevBuf par;     // concurrent Arnoldi estimates: per-iteration yk / error words, scratch and groups
  int64_t ldv = 0;
  int nl_cap = 0;
  // CUDA graph of a whole fixed-length (istop = 2) solve, replayed while the
  // launch key is unchanged
  cudaGraphExec_t graph = nullptr;
  std::vector<unsigned char> graph_key;
  int graph_kernels = 0;  // kernel nodes in the graph (launch accounting)
};

namespace psf {
// Parses fname / variant with the reference's case-sensitive, blank-padded
// comparison.  Returns false if the pair is not a valid selector.
bool parse_fun(const psfun_serial* fun, FunParams* fp);
bool fstr_eq(const char* s, const char* lit);
void set_fstr(char* dst, const char* src);  // Fortran character(len=20) assignment

int krylov_apply_device(psfun_krylov* meth, psfun_serial* fun, psfun_csr* a, double* y, const double* x, double eps,
                        int itmax, int itrace, int istop, int* iter, double* err, double* res, int res_cap,
                        int* res_len);
int serial_apply_device(psfun_serial* fun, int n, const double* a_dev, int lda, double* y_dev, const double* x_dev);
int csr_build_diag_inv(psfun_csr* a);
constexpr int kBjacRows = 32;  // rows per diagonal block of the BJAC preconditioner
int csr_build_bjac(psfun_csr* a);
// The matrix back on the host (0-based CSR).
int csr_download(psfun_csr* a, std::vector<int32_t>& irp, std::vector<int32_t>& ja, std::vector<double>& val);
int cg_device(psfun_csr* a, int prec, const double* b, double eta, double zeta, double* x, double eps, int itmax,
              int istop, int* iter, double* err, int itrace = 0, double* cond = nullptr);
int quad_apply_device(psfun_csr* a, int N, const double* xi, const double* c, double eta, double sign,
                      const double* x, double* y, double eps, int itmax, int* iter, double* err);
int spmv_device(psfun_csr* a, double alpha, const double* x, double beta, double* y);
// psfun_gpu_d_krylov_batch with KNAME 'ARNOLDI' (batch_arnoldi.cu)
int batch_arnoldi(psfun_krylov* meth, const FunParams& fp, int count, const psfun_batch_item* items, double eps,
                  int itmax, int istop, int* iters, double* errs, int* infos);
// Whether A equals A^T entry by entry (same stored pattern, equal values),
// checked once per handle on the host and cached: *sym = 1 or 0.
int csr_symmetric(psfun_csr* a, int* sym);
// A^T as a CSR handle owned by `a` (built once, on the host, rows in
// increasing column order); destroyed with `a`.
int csr_transpose(psfun_csr* a, psfun_csr** out);

// Optional per-kernel timing: CUDA events recorded around selected launches
// on the launching stream, accumulated when the solve synchronises.
enum ProfKernel { PROF_LZ_SPMV = 0, PROF_LZ_UPDATE, PROF_AR_SPMV, PROF_AR_MGS, PROF_FINAL, PROF_RECOMBINE, PROF_N };
bool prof_enabled();
void prof_begin(int kernel, cudaStream_t s);
void prof_end(int kernel, cudaStream_t s);
void prof_collect();  // call after the stream has synchronised
}  // namespace psf
