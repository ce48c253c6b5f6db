// cg.cu -- preconditioned CG for the shifted system (eta A + zeta I) x = b.
//
// Restates psfun_dcg_vect (krylov/shifted/psfun_dcg.F90:249-335) reached
// through the psb_krylov generic (krylov/psfun_krylov_mod.f90:48-142), with the
// PSBLAS stopping rule it calls (psb_init_conv / psb_check_conv /
// psb_end_conv, documented in the PSBLAS user guide):
//   istop 1: ||r||_inf <= eps * (||A||_inf ||x||_inf + ||b||_inf)
//   istop 2: ||r||_2   <= eps * ||b||_2
// and the iteration also ends once itx >= itmax.  Preconditioners: NONE and
// DIAG (Jacobi from the diagonal of A, the shifted.inp:8 choice).
//
// Per iteration three kernels: p = z + beta p; q = eta A p + zeta p with the
// fused p.q (SpMV epilogue); x += alpha p, r -= alpha q, z = D r with the fused
// r.z and the norms of the stopping rule.  Scalars (rho, sigma, alpha, beta,
// the stop test) are finalised on the device by the last block.  Iterations
// are replayed from a CUDA graph in chunks of eight.
#include <cmath>
#include <cstring>
#include <vector>

#include "internal.h"

namespace psf {

struct CgCtrl {
  int done, brk, itx, it, err, pad0;
  unsigned cnt0, cnt1;
  double rho, rho_old, sigma, alpha, beta;
  double errnum, errden;
  double bnorm_inf, bnorm2, anorm_inf;
};

struct CgState {
  int64_t n;
  int istop, itmax, prec;
  double eta, zeta, eps;
  double *x, *r, *p, *q, *z;
  const double* b;
  const double* dinv;
  double* part;   // partial sums (3 per block)
  CgCtrl* c;
  volatile int* host_flag;
};

constexpr int kCgThreads = 256;

// r = b - eta A x - zeta x ; z = D r ; rho partial (restart, :256-260)
struct EpiResid {
  const CgState* st;
  double acc;
  PSF_DEVINL void operator()(int r, double s) {
    const double v = fma(-st->zeta, st->x[r], fma(-st->eta, s, st->b[r]));
    st->r[r] = v;
    const double zz = st->dinv ? st->dinv[r] * v : v;
    st->z[r] = zz;
    acc = fma(v, zz, acc);
  }
};

__global__ void __launch_bounds__(kSpmvThreads) k_cg_restart(CgState st, CsrDev A) {
  PSF_SPMV_SMEM();
  CgCtrl* c = st.c;
  if (c->done) return;
  spmv_smem_init(sm);
  EpiResid epi{&st, 0.0};
  spmv_tiles(A, st.x, epi, sm, &c->err);
  spmv_sched_done(A);
  const double acc = block_sum(epi.acc, sm.red);
  last_block_reduce(acc, st.part, &c->cnt0, sm.red, [&](double tot) {
    c->brk = 0;
    c->it = 0;
    c->rho_old = 0.0;
    c->rho = tot;  // rho of the first iteration (r.z)
  });
}

// it += 1, itx += 1 ; p = z (it == 1) or p = z + beta p  (:267-285)
__global__ void __launch_bounds__(kCgThreads) k_cg_p(CgState st) {
  CgCtrl* c = st.c;
  if (c->done || c->brk) return;
  const int first = (c->it == 0);
  const double beta = c->beta;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < st.n; r += stride)
    st.p[r] = first ? st.z[r] : fma(beta, st.p[r], st.z[r]);
}

// q = eta A p + zeta p ; sigma = p.q ; alpha = rho/sigma  (:302-310)
__global__ void __launch_bounds__(kSpmvThreads) k_cg_q(CgState st, CsrDev A) {
  PSF_SPMV_SMEM();
  CgCtrl* c = st.c;
  if (c->done || c->brk) return;
  spmv_smem_init(sm);
  EpiShiftDot epi{st.eta, st.zeta, st.p, st.q, 0.0};
  spmv_tiles(A, st.p, epi, sm, &c->err);
  spmv_sched_done(A);
  const double acc = block_sum(epi.acc, sm.red);
  last_block_reduce(acc, st.part, &c->cnt0, sm.red, [&](double tot) {
    c->it += 1;
    c->itx += 1;
    c->sigma = tot;
    if (tot == 0.0) {
      c->brk = 1;  // sigma breakdown: exit iteration, restart
      if (st.host_flag) st.host_flag[2] = 1;
    } else {
      c->alpha = c->rho / tot;
    }
  });
}

// x += alpha p ; r -= alpha q ; z = D r ; rho' = r.z ; stop test  (:320-333)
__global__ void __launch_bounds__(kCgThreads) k_cg_xr(CgState st) {
  __shared__ double red[32];
  CgCtrl* c = st.c;
  if (c->done || c->brk) return;
  const double alpha = c->alpha;
  double a_rz = 0.0, a_r = 0.0, a_x = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < st.n; r += stride) {
    const double xv = fma(alpha, st.p[r], st.x[r]);
    st.x[r] = xv;
    const double rv = fma(-alpha, st.q[r], st.r[r]);
    st.r[r] = rv;
    const double zv = st.dinv ? st.dinv[r] * rv : rv;
    st.z[r] = zv;
    a_rz = fma(rv, zv, a_rz);
    if (st.istop == 1) {
      a_r = fmax(a_r, fabs(rv));
      a_x = fmax(a_x, fabs(xv));
    } else {
      a_r = fma(rv, rv, a_r);
    }
  }
  a_rz = block_sum(a_rz, red);
  if (st.istop == 1) {
    a_r = block_max(a_r, red);
    a_x = block_max(a_x, red);
  } else {
    a_r = block_sum(a_r, red);
  }
  __shared__ bool am_last;
  if (threadIdx.x == 0) {
    st.part[3 * blockIdx.x + 0] = a_rz;
    st.part[3 * blockIdx.x + 1] = a_r;
    st.part[3 * blockIdx.x + 2] = a_x;
    __threadfence();
    am_last = (atomicAdd(&c->cnt1, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  double s_rz = 0.0, s_r = 0.0, s_x = 0.0;
  const volatile double* pv = st.part;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    s_rz += pv[3 * b];
    if (st.istop == 1) {
      s_r = fmax(s_r, pv[3 * b + 1]);
      s_x = fmax(s_x, pv[3 * b + 2]);
    } else {
      s_r += pv[3 * b + 1];
    }
  }
  s_rz = block_sum(s_rz, red);
  if (st.istop == 1) {
    s_r = block_max(s_r, red);
    s_x = block_max(s_x, red);
  } else {
    s_r = block_sum(s_r, red);
  }
  if (threadIdx.x == 0) {
    c->cnt1 = 0u;
    double errnum, errden;
    if (st.istop == 1) {
      errnum = s_r;
      errden = c->anorm_inf * s_x + c->bnorm_inf;
    } else {
      errnum = sqrt(s_r);
      errden = c->bnorm2;
    }
    c->errnum = errnum;
    c->errden = errden;
    const bool ok = (errden == 0.0) ? (errnum <= st.eps) : (errnum <= st.eps * errden);
    if (ok || c->itx >= st.itmax) {
      c->done = 1;
      if (st.host_flag) st.host_flag[0] = 1;
    } else {
      // next iteration's rho and beta (:278-285)
      c->rho_old = c->rho;
      c->rho = s_rz;
      if (c->rho_old == 0.0) {
        c->brk = 1;  // rho breakdown at the top of the next iteration: exit it, restart
        c->itx += 1;
        if (st.host_flag) st.host_flag[2] = 1;
      } else {
        c->beta = c->rho / c->rho_old;
      }
    }
    if (st.host_flag) st.host_flag[1] = c->itx;
    __threadfence();
  }
}

// ||b||_inf, ||b||_2
__global__ void __launch_bounds__(kCgThreads) k_cg_bnorm(CgState st) {
  __shared__ double red[32];
  double a2 = 0.0, ai = 0.0;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < st.n; r += (int64_t)gridDim.x * blockDim.x) {
    const double v = st.b[r];
    a2 = fma(v, v, a2);
    ai = fmax(ai, fabs(v));
  }
  a2 = block_sum(a2, red);
  ai = block_max(ai, red);
  if (threadIdx.x == 0) {
    st.part[2 * blockIdx.x] = a2;
    st.part[2 * blockIdx.x + 1] = ai;
  }
}
__global__ void k_cg_bnorm_fin(CgState st, int nblocks) {
  __shared__ double red[32];
  double a2 = 0.0, ai = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
    a2 += st.part[2 * b];
    ai = fmax(ai, st.part[2 * b + 1]);
  }
  a2 = block_sum(a2, red);
  ai = block_max(ai, red);
  if (threadIdx.x == 0) {
    st.c->bnorm2 = sqrt(a2);
    st.c->bnorm_inf = ai;
  }
}

__global__ void k_diag_inv(int64_t n, const double* d, double* out) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
    out[r] = (d[r] != 0.0) ? 1.0 / d[r] : 1.0;
}

int cg_device(psfun_csr* a, int prec, const double* b, double eta, double zeta, double* x, double eps, int itmax,
              int istop, int* iter, double* err) {
  if (istop < 1 || istop > 2) return PSFUN_ERR_INVALID_ISTOP;
  if (!b || !x) return PSFUN_ERR_INVALID_VECT_STATE;
  const int64_t n = a->n;
  cudaStream_t s = stream();
  static DevBuf work, ctrlb, partb;
  const int64_t ld = (n + 31) & ~31LL;
  PSF_TRY(work.ensure(sizeof(double) * 4 * ld + 64));
  PSF_TRY(ctrlb.ensure(sizeof(CgCtrl) + 64));
  PSF_TRY(partb.ensure(sizeof(double) * 3 * 4096));
  if (prec == 1 && !a->diag_inv) {
    // DIAG: inverse diagonal of A (a zero diagonal entry is left as 1)
    double* dtmp = nullptr;
    PSF_CUDA(cudaMalloc(&a->diag_inv, sizeof(double) * (n + 1)));
    PSF_CUDA(cudaMalloc(&dtmp, sizeof(double) * (n + 1)));
    PSF_CUDA(cudaMemcpyAsync(dtmp, a->h_diag.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    k_diag_inv<<<256, 256, 0, s>>>(n, dtmp, a->diag_inv);
    count_launch();
    PSF_CUDA(cudaStreamSynchronize(s));
    cudaFree(dtmp);
  }
  CgState st;
  st.n = n;
  st.istop = istop;
  st.itmax = itmax;
  st.prec = prec;
  st.eta = eta;
  st.zeta = zeta;
  st.eps = eps;
  st.x = x;
  st.b = b;
  st.r = work.as<double>();
  st.p = st.r + ld;
  st.q = st.p + ld;
  st.z = st.q + ld;
  st.dinv = (prec == 1) ? a->diag_inv : nullptr;
  st.part = partb.as<double>();
  st.c = ctrlb.as<CgCtrl>();
  static volatile int* hflag = nullptr;
  static int* dflag = nullptr;
  if (!hflag) {
    int* p = nullptr;
    PSF_CUDA(cudaHostAlloc((void**)&p, 4 * sizeof(int), cudaHostAllocMapped));
    hflag = p;
    PSF_CUDA(cudaHostGetDevicePointer((void**)&dflag, p, 0));
  }
  hflag[0] = 0;
  hflag[1] = 0;
  st.host_flag = dflag;
  CgCtrl h0;
  memset(&h0, 0, sizeof h0);
  h0.anorm_inf = a->norm_inf;
  h0.errden = 1.0;
  PSF_CUDA(cudaMemcpyAsync(st.c, &h0, sizeof h0, cudaMemcpyHostToDevice, s));
  const int gv = std::max(1, std::min<int>((int)((n + kCgThreads - 1) / kCgThreads), sm_count() * 8));
  static bool attr = false;
  if (!attr) { spmv_smem_attr(k_cg_restart); spmv_smem_attr(k_cg_q); attr = true; }
  const int gs = std::max(1, std::min<int>(a->ntiles, sm_count() * 4));
  k_cg_bnorm<<<gv, kCgThreads, 0, s>>>(st);
  k_cg_bnorm_fin<<<1, kCgThreads, 0, s>>>(st, gv);
  count_launch(2);
  const CsrDev A = a->dev();
  // kCgChunk iterations (three kernels each) captured once per launch key in
  // a CUDA graph and replayed: the launch cost of the host loop is paid once
  // per chunk.  Kernels of iterations past the end return at their top.
  constexpr int kCgChunk = 8;
  struct Key {
    CgState st; CsrDev A; int gs, gv;
  } key;
  memset(&key, 0, sizeof key);
  key.st = st; key.A = A; key.gs = gs; key.gv = gv;
  static cudaGraphExec_t graph = nullptr;
  static std::vector<unsigned char> graph_key;
  const unsigned char* kb = reinterpret_cast<const unsigned char*>(&key);
  std::vector<unsigned char> kv(kb, kb + sizeof key);
  if (!graph || graph_key != kv) {
    if (graph) { cudaGraphExecDestroy(graph); graph = nullptr; }
    cudaGraph_t g = nullptr;
    PSF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < kCgChunk; ++k) {
      k_cg_p<<<gv, kCgThreads, 0, s>>>(st);
      k_cg_q<<<gs, kSpmvThreads, kSpmvSmemBytes, s>>>(st, A);
      k_cg_xr<<<gv, kCgThreads, 0, s>>>(st);
    }
    cudaError_t ec = cudaStreamEndCapture(s, &g);
    PSF_CUDA(ec);
    cudaError_t ei = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    PSF_CUDA(ei);
    graph_key = kv;
  }
  int itx_host = 0;
  while (itx_host < itmax) {  // restart loop (:252-253)
    hflag[2] = 0;
    k_cg_restart<<<gs, kSpmvThreads, kSpmvSmemBytes, s>>>(st, A);
    count_launch();
    PSF_CUDA(cudaGetLastError());
    // enqueue chunks ahead of the device; device flags end them
    for (int k = itx_host; k <= itmax + 1; k += kCgChunk) {
      if (hflag[0] || hflag[2]) break;
      PSF_CUDA(cudaGraphLaunch(graph, s));
      count_launch(3 * kCgChunk);
      for (long spin = 0; k - hflag[1] > 4 * kCgChunk && !hflag[0] && !hflag[2]; ++spin) {
        if (cudaStreamQuery(s) == cudaSuccess) break;
        if (spin > 200000000L) break;
      }
    }
    PSF_CUDA(cudaGetLastError());
    CgCtrl hc;
    PSF_CUDA(cudaMemcpyAsync(&hc, st.c, sizeof hc, cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
    if (hc.err & DEVERR_TIMEOUT) return PSFUN_ERR_DEVICE_TIMEOUT;
    itx_host = hc.itx;
    if (hc.done || !hc.brk) break;
  }
  CgCtrl hc;
  PSF_CUDA(cudaMemcpyAsync(&hc, st.c, sizeof hc, cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  if (iter) *iter = hc.itx;
  if (err) *err = (hc.errden > 0.0) ? hc.errnum / hc.errden : hc.errnum;
  return PSFUN_SUCCESS;
}

}  // namespace psf

extern "C" {

static int parse_prec(const char* ptype, int* prec) {
  std::string k(ptype ? ptype : "NONE");
  for (auto& ch : k) ch = (char)toupper((unsigned char)ch);
  while (!k.empty() && k.back() == ' ') k.pop_back();
  if (k == "NONE" || k == "NOPREC") { *prec = 0; return 1; }
  if (k == "DIAG" || k == "JACOBI") { *prec = 1; return 1; }
  return 0;
}

int psfun_gpu_dcg_device(const char* method, psfun_csr* a, const char* ptype, const double* b, double eta,
                         double zeta, double* x, double eps, int itmax, int istop, int* iter, double* err) {
  (void)method;  // only CG exists; unknown methods default to CG (psfun_krylov_mod.f90:120-125)
  if (!a) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  int prec = 0;
  if (!parse_prec(ptype, &prec)) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  return psf::cg_device(a, prec, b, eta, zeta, x, eps, itmax, istop, iter, err);
}

int psfun_gpu_dcg(const char* method, psfun_csr* a, const char* ptype, const double* b, double eta, double zeta,
                  double* x, double eps, int itmax, int istop, int* iter, double* err) {
  if (!a) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  if (!b || !x) return PSFUN_ERR_INVALID_VECT_STATE;
  const int64_t n = a->n;
  psf::DevBuf db, dx;
  PSF_TRY(db.ensure(sizeof(double) * (n + 1)));
  PSF_TRY(dx.ensure(sizeof(double) * (n + 1)));
  cudaStream_t s = psf::stream();
  PSF_CUDA(cudaMemcpyAsync(db.ptr, b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  PSF_CUDA(cudaMemcpyAsync(dx.ptr, x, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  int rc = psfun_gpu_dcg_device(method, a, ptype, db.as<double>(), eta, zeta, dx.as<double>(), eps, itmax, istop,
                                iter, err);
  if (rc == PSFUN_SUCCESS) {
    PSF_CUDA(cudaMemcpyAsync(x, dx.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    PSF_CUDA(cudaStreamSynchronize(s));
  }
  db.release();
  dx.release();
  return rc;
}

}  // extern "C"
