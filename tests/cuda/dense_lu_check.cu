// Device check of the dense solve behind the Pade step (dense.cuh::cta_lu_solve):
// A X = B with partial pivoting on one block and on a cooperative group of 8
// (the substitutions shared), for orders on both sides of the one-barrier
// factorisation's limit (128), on matrices that pivot at most steps.  For each
// case it prints
//   case <name> m <m> G <G> ok <0|1> berr <normwise backward error> pivdiff <n>
// where pivdiff counts the steps whose pivot row differs from a host
// elimination with IDAMAX's rule (first row of largest magnitude).
// Built and run by tests/test_gpu_dense_lu.py.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <cuda_runtime.h>

#include "internal.h"
#include "dense.cuh"

using namespace psf;

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_lu(int m, int nrhs, double* A, double* B, double* ws, int* ok,
                                                 DenseGroup* grp) {
  if (blockIdx.x > 0) {
    dense_helper(grp);
    return;
  }
  __shared__ DenseSmem sm;
  dense_group_begin(sm, grp);
  const bool r = cta_lu_solve(m, nrhs, A, m, B, m, ws, sm);
  if (threadIdx.x == 0) *ok = r ? 1 : 0;
  dense_group_end(sm, ok + 1);
}

struct Rng {
  unsigned long long s;
  double next() {  // uniform in [-0.5, 0.5)
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    return (double)(s >> 11) / 9007199254740992.0 - 0.5;
  }
};

// pivot rows of an elimination with partial pivoting (IDAMAX: first maximum)
static std::vector<int> host_pivots(int m, std::vector<double> a) {
  std::vector<int> piv(m);
  for (int k = 0; k < m; ++k) {
    int p = k;
    double best = std::fabs(a[k + (size_t)k * m]);
    for (int i = k + 1; i < m; ++i)
      if (std::fabs(a[i + (size_t)k * m]) > best) { best = std::fabs(a[i + (size_t)k * m]); p = i; }
    piv[k] = p;
    if (best == 0.0) break;
    for (int j = k; j < m; ++j) std::swap(a[k + (size_t)j * m], a[p + (size_t)j * m]);
    const double r = 1.0 / a[k + (size_t)k * m];
    for (int i = k + 1; i < m; ++i) a[i + (size_t)k * m] *= r;
    for (int j = k + 1; j < m; ++j)
      for (int i = k + 1; i < m; ++i)
        a[i + (size_t)j * m] = std::fma(-a[i + (size_t)k * m], a[k + (size_t)j * m], a[i + (size_t)j * m]);
  }
  return piv;
}

static int run_case(const char* name, int m, int G, const std::vector<double>& a, const std::vector<double>& b,
                    int nrhs, bool singular) {
  const size_t mm = (size_t)m * m, mb = (size_t)m * nrhs;
  double *A = nullptr, *B = nullptr, *W = nullptr;
  int* ok = nullptr;
  DenseGroup* g = nullptr;
  if (cudaMalloc(&A, 8 * mm) || cudaMalloc(&B, 8 * mb) || cudaMalloc(&W, 8 * (2 * (size_t)m + 64)) ||
      cudaMalloc(&ok, 8) || cudaMalloc(&g, sizeof(DenseGroup) + 64)) {
    printf("cuda malloc failed\n");
    return 1;
  }
  cudaMemset(g, 0, sizeof(DenseGroup));
  cudaMemset(ok, 0, 8);
  cudaMemcpy(A, a.data(), 8 * mm, cudaMemcpyHostToDevice);
  cudaMemcpy(B, b.data(), 8 * mb, cudaMemcpyHostToDevice);
  DenseGroup* gp = (G > 1) ? g : nullptr;
  void* args[] = {&m, &nrhs, &A, &B, &W, &ok, &gp};
  cudaError_t e = cudaLaunchCooperativeKernel((void*)k_lu, dim3(G), dim3(kThreads), args, 0, 0);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    printf("cuda error %s\n", cudaGetErrorString(e));
    return 1;
  }
  int hok[2] = {0, 0};
  std::vector<double> x(mb), ws(2 * (size_t)m + 64);
  cudaMemcpy(hok, ok, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(x.data(), B, 8 * mb, cudaMemcpyDeviceToHost);
  cudaMemcpy(ws.data(), W, 8 * ws.size(), cudaMemcpyDeviceToHost);
  cudaFree(A); cudaFree(B); cudaFree(W); cudaFree(ok); cudaFree(g);
  double berr = 0.0;
  int pivdiff = 0;
  if (hok[0] && !singular) {
    double anorm = 0.0;
    for (int i = 0; i < m; ++i) {
      double s = 0.0;
      for (int j = 0; j < m; ++j) s += std::fabs(a[i + (size_t)j * m]);
      anorm = std::fmax(anorm, s);
    }
    for (int c = 0; c < nrhs; ++c) {
      double rmax = 0.0, xmax = 0.0, bmax = 0.0;
      for (int i = 0; i < m; ++i) {
        long double r = -(long double)b[i + (size_t)c * m];
        for (int j = 0; j < m; ++j) r += (long double)a[i + (size_t)j * m] * x[j + (size_t)c * m];
        rmax = std::fmax(rmax, std::fabs((double)r));
        xmax = std::fmax(xmax, std::fabs(x[i + (size_t)c * m]));
        bmax = std::fmax(bmax, std::fabs(b[i + (size_t)c * m]));
      }
      berr = std::fmax(berr, rmax / (anorm * xmax + bmax));
    }
    const std::vector<int> hp = host_pivots(m, a);
    const int* dp = reinterpret_cast<const int*>(ws.data());
    for (int k = 0; k < m; ++k) pivdiff += (dp[k] != hp[k]);
  }
  printf("case %s m %d G %d ok %d berr %.3e pivdiff %d grouperr %d\n", name, m, G, hok[0], berr, pivdiff, hok[1]);
  return 0;
}

int main() {
  int rc = 0;
  for (int m : {1, 2, 3, 5, 17, 31, 33, 64, 80, 127, 128, 129, 150}) {
    for (int G : {1, 8}) {
      Rng r{0x9E3779B97F4A7C15ULL ^ (unsigned long long)(m * 131 + G)};
      const size_t mm = (size_t)m * m;
      std::vector<double> a(mm), b(mm);
      // random: pivots at most steps
      for (auto& v : a) v = r.next();
      for (auto& v : b) v = r.next();
      rc |= run_case("random", m, G, a, b, m, false);
      // reversed dominant anti-diagonal: every step exchanges rows
      for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) a[i + (size_t)j * m] = 0.01 * r.next() + ((i + j == m - 1) ? 1.0 + 0.1 * r.next() : 0.0);
      rc |= run_case("antidiag", m, G, a, b, 3 < m ? 3 : m, false);
      // one zero column: an exactly zero pivot, reported as singular
      if (m >= 5) {
        for (auto& v : a) v = r.next();
        for (int i = 0; i < m; ++i) a[i + (size_t)3 * m] = 0.0;
        rc |= run_case("singular", m, G, a, b, m, true);
      }
    }
  }
  return rc;
}
