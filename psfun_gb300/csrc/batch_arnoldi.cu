// batch_arnoldi.cu -- Arnoldi f(tA)x for many instances and right-hand sides
// at once (psfun_gpu_d_krylov_batch with KNAME 'ARNOLDI').
//
// Every (instance, right-hand side) pair is a unit that follows the control
// flow of psfun_d_arnoldi (krylov/polynomial/psfun_d_arnoldi.f90:98-343) on
// the Krylov space of t A (the item's scaling t in the role of fun%scaling):
// W_i = t A v_{i-1}, modified Gram-Schmidt against v_1..v_{i-1} (:210-217),
// h(i,i-1) = ||w||, the a posteriori estimate of istop = 1 (:222-276) with
// the dense f of the function object, the final f on H(1:itx-1) when no
// estimate converged (:282-314) and the assembly of the first coefficients
// (:325-329).  As in the single-pair path, the basis slots hold W_k unscaled
// with s_k = 1 / ||W_k|| kept apart.
//
// One Arnoldi step of every unit is one cooperative launch (k_ba_step): the
// grid's blocks are partitioned among the units in proportion to their rows,
// every block forms the SpMV and the Gram-Schmidt sweeps of its unit's rows,
// and one bounded grid barrier per sweep serves all units (the units are at
// the same step).  Each unit's dot products are the sums of its blocks'
// partials in block order, formed by every block of the unit alike, so the
// results are reproducible.  The per-pair estimates run one block per unit
// (k_ba_estimate) and a one-block kernel advances the device step counter and
// counts the live units (k_ba_next).  The three kernels of a step read the
// step from device memory, so they are captured once per call as a CUDA
// graph and the graph is replayed for every step.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace psf {

constexpr int kBaThreads = 256;

// One (instance, right-hand side) pair.
struct BaUnit {
  CsrDev A;
  int64_t n, ldv;
  double t;
  double* V;     // (nl+1) slots of ldv
  double* H;     // (nl+1)^2, column-major, the reference's h
  double* s;     // nl + 2: s_k = 1 / ||W_k||
  double* rs;    // nl + 2: rs(1) = beta0, rs(i) the estimates
  double* yk;    // nl + 2
  double* coef;  // nl + 2
  double* scr;   // dense f(H) scratch
  const double* x;
  double* y;
  int b0, b1;  // blocks of the step kernel
  int done, conv, breakdown, itx, yk_len, nterms, info, pad;
  double beta0, errnum, errden;
};

struct BaArgs {
  BaUnit* u;
  int count, nl, ldh, istop, keeplast;
  double eps;
  FunParams fp;
  const int* blk_unit;  // unit of every block of the step kernel
  double* part;         // 4 x gridDim.x partial sums
  unsigned* bar;        // grid barrier counter, zeroed before every step
  int* err;
  int* step;            // the current step i
  const double* e1;     // nl + 2: e1
  volatile int* host_flag;  // mapped: [0] live units, [1] last step done
};

#define BH(U, ldh, i, j) (U).H[((i)-1) + (size_t)((j)-1) * (ldh)]
#define BW(U, k) ((U).V + (size_t)((k)-1) * (U).ldv)

// Rows [r0, r1) of unit u that block b works on.
PSF_DEVINL void ba_rows(const BaUnit& U, int b, int64_t* r0, int64_t* r1) {
  const int nb = U.b1 - U.b0, k = b - U.b0;
  const int64_t per = (U.n + nb - 1) / nb;
  *r0 = min(U.n, (int64_t)k * per);
  *r1 = min(U.n, *r0 + per);
}

// Sum of the partials of the unit's blocks, in block order (every thread).
PSF_DEVINL double ba_unit_sum(const double* part, const BaUnit& U, double* red) {
  return block_sum_array(part + U.b0, U.b1 - U.b0, red);
}

// W_1 = x, beta0 = ||x||, s_1 = 1 / beta0   (psfun_d_arnoldi.f90:183-197)
__global__ void __launch_bounds__(kBaThreads) k_ba_init(BaArgs B) {
  __shared__ double red[32];
  const int b = blockIdx.x;
  BaUnit& U = B.u[B.blk_unit[b]];
  int64_t r0, r1;
  ba_rows(U, b, &r0, &r1);
  double acc = 0.0;
  double* w1 = BW(U, 1);
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const double v = U.x[r];
    w1[r] = v;
    acc = fma(v, v, acc);
  }
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) B.part[b] = acc;
  if (!grid_sync_to(B.bar, (unsigned)gridDim.x, B.err)) return;
  const double tot = ba_unit_sum(B.part, U, red);
  if (b == U.b0 && threadIdx.x == 0) {
    const double b0 = sqrt(tot);
    U.beta0 = b0;
    U.rs[0] = b0;
    U.errnum = 0.0;
    U.errden = 1.0;
    if (b0 == 0.0) {
      U.done = 1;
      U.itx = 0;
    } else {
      U.s[1] = 1.0 / b0;
    }
  }
}

// Step i of every live unit: W_i = t s_{i-1} A W_{i-1} with the dots of
// its rows with W_1 and W_2 formed as they are computed, then Gram-Schmidt
// against W_1..W_{i-1} taking the basis vectors two at a time as the plain
// Arnoldi kernel does (one sweep subtracts h(k) v_k and h(k+1) v_{k+1} and
// forms the dots with v_{k+2} and v_{k+3}, or the norm; h(k+1) is taken from
// w before the v_k update), then h(i,i-1) and s_i.  One grid barrier per
// pair of vectors serves all units.  Units that have stopped only keep the
// barriers.
__global__ void __launch_bounds__(kBaThreads) k_ba_step(BaArgs B) {
  __shared__ double red[32];
  __shared__ double sc[2];
  const int i = *B.step;
  if (i > B.nl) return;
  const int b = blockIdx.x, G = gridDim.x;
  BaUnit& U = B.u[B.blk_unit[b]];
  const bool live = !U.done;
  int64_t r0, r1;
  ba_rows(U, b, &r0, &r1);
  const int ldh = B.ldh;
  const int nv = i - 1;
  double* w = BW(U, i);
  unsigned nb = 0;
  auto gsync = [&]() { return grid_sync_to(B.bar, (++nb) * (unsigned)G, B.err); };
  // partials: two buffers of two values per block (value q of buffer p at
  // part[(2 p + q) G + b])
  auto put2 = [&](int p, double a1, double a2, bool two) {
    a1 = block_sum(a1, red);
    if (two) a2 = block_sum(a2, red);
    if (threadIdx.x == 0) {
      B.part[(size_t)(2 * p) * G + b] = a1;
      if (two) B.part[(size_t)(2 * p + 1) * G + b] = a2;
    }
  };
  {  // SpMV of the unit's rows, with the dots of w with W_1 and W_2
    double acc1 = 0.0, acc2 = 0.0;
    if (live) {
      const double f = U.t * U.s[i - 1];
      const double* wp = BW(U, i - 1);
      const double* w1 = BW(U, 1);
      const double* w2 = BW(U, nv >= 2 ? 2 : 1);
      for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        double acc = 0.0;
        for (int k = U.A.irp[r], ke = U.A.irp[r + 1]; k < ke; ++k) acc = fma(U.A.val[k], __ldg(wp + U.A.ja[k]), acc);
        const double v = f * acc;
        w[r] = v;
        acc1 = fma(w1[r], v, acc1);
        if (nv >= 2) acc2 = fma(w2[r], v, acc2);
      }
    }
    put2(0, acc1, acc2, nv >= 2);
  }
  if (!gsync()) return;
  int buf = 0;
  for (int k = 1; k <= nv; k += 2) {
    const bool two = k + 1 <= nv;
    const int kn = k + 2;
    const int next = (kn > nv) ? 0 : ((kn + 1 <= nv) ? 2 : 1);
    const double t1 = ba_unit_sum(B.part + (size_t)(2 * buf) * G, U, red);
    const double t2 = two ? ba_unit_sum(B.part + (size_t)(2 * buf + 1) * G, U, red) : 0.0;
    if (threadIdx.x == 0) {
      const double h1 = U.s[k] * t1;  // h(k,i-1) = v_k . w
      if (live && b == U.b0) BH(U, ldh, k, i - 1) = h1;
      sc[0] = h1 * U.s[k];
      if (two) {
        const double h2 = U.s[k + 1] * t2;
        if (live && b == U.b0) BH(U, ldh, k + 1, i - 1) = h2;
        sc[1] = h2 * U.s[k + 1];
      }
    }
    __syncthreads();
    const double c1 = sc[0], c2 = two ? sc[1] : 0.0;
    double acc1 = 0.0, acc2 = 0.0;
    if (live) {
      const double* wk = BW(U, k);
      const double* wk1 = BW(U, two ? k + 1 : k);
      const double* wn1 = BW(U, next >= 1 ? kn : k);
      const double* wn2 = BW(U, next == 2 ? kn + 1 : k);
      for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
        double v = fma(-c1, wk[r], w[r]);
        if (two) v = fma(-c2, wk1[r], v);
        w[r] = v;
        if (next == 0) {
          acc1 = fma(v, v, acc1);
        } else {
          acc1 = fma(wn1[r], v, acc1);
          if (next == 2) acc2 = fma(wn2[r], v, acc2);
        }
      }
    }
    buf ^= 1;
    put2(buf, acc1, acc2, next == 2);
    if (!gsync()) return;
  }
  const double tot = ba_unit_sum(B.part + (size_t)(2 * buf) * G, U, red);
  if (live && b == U.b0 && threadIdx.x == 0) {
    const double beta = sqrt(tot);
    BH(U, ldh, i, i - 1) = beta;
    U.s[i] = 1.0 / beta;
    U.itx = i - 1;
    if (beta == 0.0) {  // invariant subspace: the unit stops here
      U.breakdown = 1;
      U.done = 1;
    }
  }
}

// The a posteriori estimate of iteration i of every live unit, one block per
// unit: yk = f(H(1:i-1,1:i-1)) e1, rs(i) = beta0 h(i,i-1) |yk(i-1)| / ||yk||.
__global__ void __launch_bounds__(kBaThreads) k_ba_estimate(BaArgs B) {
  __shared__ DenseSmem sm;
  const int i = *B.step;
  BaUnit& U = B.u[blockIdx.x];
  if (i > B.nl || U.done) return;
  dense_group_begin(sm, nullptr);
  dense_use_dynamic_smem(sm);
  if (B.istop != 1) {
    if (i == B.nl && threadIdx.x == 0) U.done = 1;  // the loop ends after iteration nl
    return;
  }
  const int m = i - 1;
  const int rc = fh_apply_cta(B.fp, m, U.H, B.ldh, B.e1, U.yk, U.scr, false, sm);
  if (rc) {
    if (threadIdx.x == 0) {
      U.info = PSFUN_ERR_FROM_SUBROUTINE_NON;
      U.done = 1;
    }
    return;
  }
  double ss = 0.0;
  for (int j = threadIdx.x; j < m; j += blockDim.x) ss = fma(U.yk[j], U.yk[j], ss);
  ss = block_sum(ss, sm.red);
  if (threadIdx.x == 0) {
    const double errnum = U.beta0 * BH(U, B.ldh, i, i - 1) * fabs(U.yk[m - 1]);
    const double errden = sqrt(ss);
    const double r = errnum / errden;
    U.rs[i - 1] = r;
    U.errnum = errnum;
    U.errden = errden;
    if (r < B.eps) {
      U.conv = 1;
      U.done = 1;
      U.yk_len = m;
      U.itx = i - 1;
    } else if (i == B.nl) {
      U.done = 1;
    }
  }
}

// Advances the step and reports the live units to the host.
__global__ void k_ba_next(BaArgs B) {
  __shared__ double red[32];
  double live = 0.0;
  for (int k = threadIdx.x; k < B.count; k += blockDim.x) live += B.u[k].done ? 0.0 : 1.0;
  live = block_sum(live, red);
  if (threadIdx.x == 0) {
    const int i = *B.step;
    *B.step = i + 1;
    if (B.host_flag) {
      B.host_flag[0] = (int)live;
      B.host_flag[1] = i;
    }
  }
}

// Final f when no estimate converged and the assembly coefficients
// (psfun_d_arnoldi.f90:282-329), one block per unit.
__global__ void __launch_bounds__(kBaThreads) k_ba_final(BaArgs B) {
  __shared__ DenseSmem sm;
  BaUnit& U = B.u[blockIdx.x];
  dense_group_begin(sm, nullptr);
  dense_use_dynamic_smem(sm);
  if (U.info != 0) return;
  if (U.beta0 == 0.0) {
    if (threadIdx.x == 0) { U.nterms = 0; U.itx = 0; }
    return;
  }
  int yk_len = U.yk_len;
  if (!U.conv) {
    const int m = U.breakdown ? U.itx : U.itx - 1;
    if (m < 1) {
      if (threadIdx.x == 0) U.info = PSFUN_ERR_FROM_SUBROUTINE_NON;
      return;
    }
    const int rc = fh_apply_cta(B.fp, m, U.H, B.ldh, B.e1, U.yk, U.scr, false, sm);
    if (rc) {
      if (threadIdx.x == 0) U.info = PSFUN_ERR_FROM_SUBROUTINE_NON;
      return;
    }
    yk_len = m;
  }
  int nterms = (U.conv && !B.keeplast) ? max(U.itx - 1, 1) : yk_len;
  nterms = min(nterms, yk_len);
  for (int j = threadIdx.x; j < nterms; j += blockDim.x) U.coef[j] = U.beta0 * U.yk[j] * U.s[j + 1];
  __syncthreads();
  if (threadIdx.x == 0) {
    U.yk_len = yk_len;
    U.nterms = nterms;
  }
}

// y = sum_j coef_j W_{j+1} on the unit's rows (the step kernel's partition).
__global__ void __launch_bounds__(kBaThreads) k_ba_recombine(BaArgs B) {
  const int b = blockIdx.x;
  const BaUnit& U = B.u[B.blk_unit[b]];
  int64_t r0, r1;
  ba_rows(U, b, &r0, &r1);
  const int nt = (U.info == 0) ? U.nterms : 0;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    double acc = 0.0;
    for (int j = 0; j < nt; ++j) acc = fma(U.coef[j], U.V[(size_t)j * U.ldv + r], acc);
    U.y[r] = acc;
  }
}

// One psfun_gpu_d_krylov_batch call with KNAME 'ARNOLDI'.
int batch_arnoldi(psfun_krylov* meth, const FunParams& fp_in, int count, const psfun_batch_item* items, double eps,
                  int itmax, int istop, int* iters, double* errs, int* infos) {
  const int R = items[0].nrhs;
  const int nu = count * R;
  const int nl = itmax;
  const int ldh = nl + 1;
  FunParams fp = fp_in;
  fp.scaling = 1.0;  // the Krylov space carries the item's scaling
  cudaStream_t s = stream();
  // the step kernel's grid: every block co-resident, at least one per unit
  static int per = 0;
  if (!per) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_ba_step, kBaThreads, 0);
    if (per < 1) per = 1;
  }
  const int gmax = sm_count() * per;
  if (nu > gmax) {
    set_last_error("batched Arnoldi: " + std::to_string(nu) + " pairs exceed the " + std::to_string(gmax) +
                   " co-resident blocks of one launch");
    return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  }
  std::vector<BaUnit> hu(nu);
  int64_t rows = 0, nmax = 0;
  for (int k = 0; k < count; ++k) {
    rows += items[k].a->n * R;
    nmax = std::max<int64_t>(nmax, items[k].a->n);
  }
  // Blocks of the step kernel per unit: in proportion to the rows, at least
  // one per unit, at most gmax in all, and no fewer than `rpb` rows per block.
  // More blocks bring more of the GPU to a sweep; fewer make each sweep's grid
  // barrier cheaper.  rpb is chosen by timing the first steps once per batch shape.
  std::vector<int> nblk(nu);
  auto partition = [&](int rpb) {
    int G = 0;
    for (int k = 0; k < count; ++k)
      for (int q = 0; q < R; ++q) {
        const int64_t n = items[k].a->n;
        int nbk = (int)std::max<int64_t>(
            1, (int64_t)((double)(gmax - nu) * (double)n / (double)std::max<int64_t>(rows, 1)));
        nbk = (int)std::min<int64_t>(nbk, std::max<int64_t>(1, (n + rpb - 1) / rpb));
        nblk[k * R + q] = nbk;
        G += nbk;
      }
    while (G > gmax) {  // rounding left too many: take from the largest
      int big = (int)(std::max_element(nblk.begin(), nblk.end()) - nblk.begin());
      if (nblk[big] <= 1) break;
      --nblk[big];
      --G;
    }
    return G;
  };
  // workspace: one allocation, carved per unit at 256-byte boundaries
  size_t off = 0;
  auto carve = [&](size_t doubles) {
    const size_t o = off;
    off += (doubles + 31) & ~(size_t)31;
    return o;
  };
  const size_t fsz = fh_scratch_doubles(nl + 1, fp.phiorder) + 64;
  // a unit's dense evaluations keep their Pade work matrices in shared
  // memory when those of the largest order fit
  size_t dsmem = 0;
  if (fh_uses_gemm(fp)) {
    const size_t M = (size_t)nl + 1 + (fp.fname == FN_PHI ? (size_t)std::max(fp.phiorder, 1) : 0);
    const size_t want = sizeof(double) * ((fp.fname == FN_PHI ? 6 : 5) * M * M + 64);
    if (want <= (size_t)200 * 1024 &&
        cudaFuncSetAttribute(k_ba_estimate, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want) == cudaSuccess &&
        cudaFuncSetAttribute(k_ba_final, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)want) == cudaSuccess)
      dsmem = want;
    (void)cudaGetLastError();
  }
  struct Off { size_t V, H, s, rs, yk, coef, scr; };
  std::vector<Off> uo(nu);
  for (int u = 0; u < nu; ++u) {
    const psfun_csr* a = items[u / R].a;
    const int64_t ldv = (a->n + 31) & ~(int64_t)31;
    uo[u].V = carve((size_t)(nl + 1) * ldv);
    uo[u].H = carve((size_t)ldh * ldh);
    uo[u].s = carve(nl + 2);
    uo[u].rs = carve(nl + 2);
    uo[u].yk = carve(nl + 2);
    uo[u].coef = carve(nl + 2);
    uo[u].scr = carve(fsz);
  }
  const size_t oUnits = carve((sizeof(BaUnit) * nu + 7) / 8);
  const size_t oPart = carve(4 * (size_t)gmax + 8);
  const size_t oMap = carve(((size_t)gmax + 1) / 2 + 1);
  const size_t oE1 = carve(nl + 2);
  const size_t oMisc = carve(8);
  DevBuf& ws = meth->scratch;  // the method handle's scratch, reused for the batch
  PSF_TRY(ws.ensure(sizeof(double) * off));
  double* base = ws.as<double>();
  // One solve with the partition of rpb (a tuning run stops after
  // tune_steps steps and reports the time of its steps in *tune_ms).
  auto solve = [&](int rpb, int tune_steps, float* tune_ms) -> int {
    const int G = partition(rpb);
    int b = 0;
    std::vector<int> blk_unit(G);
    for (int u = 0; u < nu; ++u) {
      const int k = u / R, q = u % R;
      const psfun_csr* a = items[k].a;
      BaUnit& U = hu[u];
      memset(&U, 0, sizeof U);
      U.A = a->dev();
      U.n = a->n;
      U.ldv = (a->n + 31) & ~(int64_t)31;
      U.t = items[k].scaling;
      U.V = base + uo[u].V;
      U.H = base + uo[u].H;
      U.s = base + uo[u].s;
      U.rs = base + uo[u].rs;
      U.yk = base + uo[u].yk;
      U.coef = base + uo[u].coef;
      U.scr = base + uo[u].scr;
      U.x = items[k].x + (size_t)q * a->n;
      U.y = items[k].y + (size_t)q * a->n;
      U.b0 = b;
      U.b1 = b + nblk[u];
      for (int j = U.b0; j < U.b1; ++j) blk_unit[j] = u;
      b = U.b1;
      PSF_CUDA(cudaMemsetAsync(U.H, 0, sizeof(double) * (size_t)ldh * ldh, s));
      PSF_CUDA(cudaMemsetAsync(U.s, 0, sizeof(double) * 4 * ((nl + 2 + 31) & ~31), s));
    }
    BaUnit* du = reinterpret_cast<BaUnit*>(base + oUnits);
    PSF_CUDA(cudaMemcpyAsync(du, hu.data(), sizeof(BaUnit) * nu, cudaMemcpyHostToDevice, s));
    int* dmap = reinterpret_cast<int*>(base + oMap);
    PSF_CUDA(cudaMemcpyAsync(dmap, blk_unit.data(), sizeof(int) * G, cudaMemcpyHostToDevice, s));
    std::vector<double> e1(nl + 2, 0.0);
    e1[0] = 1.0;
    PSF_CUDA(cudaMemcpyAsync(base + oE1, e1.data(), sizeof(double) * (nl + 2), cudaMemcpyHostToDevice, s));
    unsigned* misc = reinterpret_cast<unsigned*>(base + oMisc);
    PSF_CUDA(cudaMemsetAsync(misc, 0, sizeof(double) * 8, s));
    static volatile int* hflag = nullptr;
    static int* dflag = nullptr;
    if (!hflag) {
      int* p = nullptr;
      PSF_CUDA(cudaHostAlloc((void**)&p, 4 * sizeof(int), cudaHostAllocMapped));
      hflag = p;
      PSF_CUDA(cudaHostGetDevicePointer((void**)&dflag, p, 0));
    }
    hflag[0] = nu;
    hflag[1] = 0;
    BaArgs B;
    B.u = du;
    B.count = nu;
    B.nl = nl;
    B.ldh = ldh;
    B.istop = istop;
    B.keeplast = meth->keeplast;
    B.eps = eps;
    B.fp = fp;
    B.blk_unit = dmap;
    B.part = base + oPart;
    B.bar = misc;
    B.err = reinterpret_cast<int*>(misc + 1);
    B.step = reinterpret_cast<int*>(misc + 2);
    B.e1 = base + oE1;
    B.host_flag = dflag;
    const int two = 2;
    PSF_CUDA(cudaMemcpyAsync(B.step, &two, sizeof(int), cudaMemcpyHostToDevice, s));
    {
      void* args[] = {(void*)&B};
      PSF_CUDA(cudaLaunchCooperativeKernel((void*)k_ba_init, dim3(G), dim3(kBaThreads), args, 0, s));
      count_launch();
    }
    // one Arnoldi step of every unit, captured once and replayed
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    {
      PSF_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      void* args[] = {(void*)&B};
      cudaError_t e = cudaMemsetAsync(B.bar, 0, sizeof(unsigned), s);
      if (e == cudaSuccess)
        e = cudaLaunchCooperativeKernel((void*)k_ba_step, dim3(G), dim3(kBaThreads), args, 0, s);
      if (e == cudaSuccess) e = cudaLaunchKernel((void*)k_ba_estimate, dim3(nu), dim3(kBaThreads), args, dsmem, s);
      if (e == cudaSuccess) e = cudaLaunchKernel((void*)k_ba_next, dim3(1), dim3(256), args, 0, s);
      cudaError_t ec = cudaStreamEndCapture(s, &graph);
      if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        PSF_CUDA(e);
      }
      PSF_CUDA(ec);
      cudaError_t ei = cudaGraphInstantiate(&gexec, graph, 0);
      cudaGraphDestroy(graph);
      PSF_CUDA(ei);
    }
    const int max_ahead = 3;
    int rc = PSFUN_SUCCESS;
    static cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (tune_steps > 0) {
      if (!ev0) {
        PSF_CUDA(cudaEventCreate(&ev0));
        PSF_CUDA(cudaEventCreate(&ev1));
      }
      PSF_CUDA(cudaEventRecord(ev0, s));
    }
    const int i_stop = (tune_steps > 0) ? std::min(nl, 1 + tune_steps) : nl;
    for (int i = 2; i <= i_stop; ++i) {
      if (hflag[0] == 0) break;  // every unit has stopped
      cudaError_t e = cudaGraphLaunch(gexec, s);
      if (e != cudaSuccess) {
        (void)cudaGetLastError();
        set_last_error(std::string("batched Arnoldi: cudaGraphLaunch: ") + cudaGetErrorString(e));
        rc = PSFUN_ERR_CUDA;
        break;
      }
      count_launch(3);
      for (long spin = 0; i - hflag[1] > max_ahead && hflag[0] != 0; ++spin) {
        if (cudaStreamQuery(s) == cudaSuccess) break;
        if (spin > 200000000L) break;
      }
    }
    cudaGraphExecDestroy(gexec);
    PSF_TRY(rc);
    if (tune_steps > 0) {
      PSF_CUDA(cudaEventRecord(ev1, s));
      PSF_CUDA(cudaEventSynchronize(ev1));
      PSF_CUDA(cudaEventElapsedTime(tune_ms, ev0, ev1));
      return PSFUN_SUCCESS;
    }
    {
      void* args[] = {(void*)&B};
      PSF_CUDA(cudaLaunchKernel((void*)k_ba_final, dim3(nu), dim3(kBaThreads), args, dsmem, s));
      PSF_CUDA(cudaLaunchKernel((void*)k_ba_recombine, dim3(G), dim3(kBaThreads), args, 0, s));
      count_launch(2);
    }
    return PSFUN_SUCCESS;
  };

  // rows per block: timed once per batch shape (count, pairs, size buckets)
  static std::vector<std::pair<std::vector<int64_t>, int>> tuned;
  auto bucket = [](int64_t v) { int b = 0; while (v > 1) { v >>= 1; ++b; } return (int64_t)b; };
  const std::vector<int64_t> key = {count, R, bucket(rows), bucket(nmax), bucket(nl), (int64_t)fp.fname,
                                    (int64_t)fp.variant};
  int rpb = 0;
  for (const auto& t : tuned)
    if (t.first == key) rpb = t.second;
  if (!rpb) {
    const int cand[] = {64, 256, 1024, 4096};
    float best = 0.0f;
    for (int c : cand) {
      float ms = 0.0f;
      PSF_TRY(solve(c, std::min(8, nl - 1), &ms));
      if (!rpb || ms < best) { best = ms; rpb = c; }
    }
    tuned.emplace_back(key, rpb);
  }
  PSF_TRY(solve(rpb, 0, nullptr));
  int herr = 0;
  PSF_CUDA(cudaMemcpyAsync(&herr, reinterpret_cast<unsigned*>(base + oMisc) + 1, sizeof(int),
                           cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaMemcpyAsync(hu.data(), base + oUnits, sizeof(BaUnit) * nu, cudaMemcpyDeviceToHost, s));
  PSF_CUDA(cudaStreamSynchronize(s));
  if (herr & DEVERR_TIMEOUT) {
    set_last_error("device-side wait timed out");
    return PSFUN_ERR_DEVICE_TIMEOUT;
  }
  int worst = PSFUN_SUCCESS;
  for (int u = 0; u < nu; ++u) {
    const BaUnit& U = hu[u];
    if (iters) iters[u] = U.conv ? U.yk_len : U.itx;
    if (errs) errs[u] = (U.errden > 0.0) ? U.errnum / U.errden : U.errnum;
    if (infos) infos[u] = U.info;
    if (U.info && worst == PSFUN_SUCCESS) worst = U.info;
  }
  return worst;
}

}  // namespace psf
