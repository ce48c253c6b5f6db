// quadrule.cpp -- host side of the rational quadrature: the Hale-Higham-
// Trefethen conformal-map rule and the elliptic functions it needs.
//
// Restates, in C++ std::complex<double>:
//   ellipkkp   utils/psfun_d_utils_mod.f90:37-99    (AGM to machine epsilon)
//   d_ellipj   utils/psfun_d_utils_mod.f90:101-117  (Bulirsch sn/cn/dn, the
//              algorithm of the vendored sncndn, elliptic_integral.f90:5089)
//   z_ellipj   utils/psfun_z_utils_mod.f90:39-107   (descending Landen)
//   horner     utils/psfun_d_utils_mod.f90:119-138
//   hhtmethod1 quadratures/psfun_z_quadrules_mod.f90:40-85
// These run once per quadrature set-up on O(N) scalars; the shifted solves
// that consume the poles and weights run on the GPU.
#include <cfloat>
#include <cmath>
#include <complex>

#include "../../include/psfun_gb300.h"

namespace {

using zd = std::complex<double>;
const double kPi = 3.14159265358979323846264338327950288;

void ellipkkp(double L, double* K) {
  if (L > 10.0) {
    K[0] = kPi / 2.0;
    K[1] = kPi * L + std::log(4.0);
    return;
  }
  const double M = std::exp(-2.0 * kPi * L);
  for (int pass = 0; pass < 2; ++pass) {
    double a0 = 1.0, b0 = std::sqrt(pass == 0 ? 1.0 - M : M), a1 = 1.0, mm = 1.0;
    int i1 = 0;
    while (mm > DBL_EPSILON) {
      a1 = (a0 + b0) / 2.0;
      const double b1 = std::sqrt(a0 * b0);
      const double c1 = (a0 - b0) / 2.0;
      ++i1;
      mm = std::ldexp(1.0, i1) * (c1 * c1);
      a0 = a1;
      b0 = b1;
    }
    K[pass] = kPi / (2.0 * a1);
  }
}

// Bulirsch (Numer. Math. 7 (1965) 78-90): descending Gauss transformation.
void sncndn(double u, double m, double* sn, double* cn, double* dn) {
  double mc = 1.0 - m, uu = u, d = 1.0;
  if (mc == 0.0) {
    *cn = 1.0 / std::cosh(uu);
    *dn = *cn;
    *sn = std::tanh(uu);
    return;
  }
  if (m > 1.0) {
    d = 1.0 - mc;
    mc = -mc / d;
    d = std::sqrt(d);
    uu = d * uu;
  }
  const double ca = std::sqrt(DBL_EPSILON);
  double a = 1.0, c = 0.0, dv = 1.0;
  double am[25], an[25];
  int l = 25;
  for (int i = 0; i < 25; ++i) {
    am[i] = a;
    mc = std::sqrt(mc);
    an[i] = mc;
    c = 0.5 * (a + mc);
    if (std::fabs(a - mc) <= ca * a) {
      l = i + 1;
      break;
    }
    mc = a * mc;
    a = c;
  }
  uu = c * uu;
  double s = std::sin(uu), co = std::cos(uu);
  if (s != 0.0) {
    a = co / s;
    c = a * c;
    for (int i = l - 1; i >= 0; --i) {
      const double b = am[i];
      a = c * a;
      c = dv * c;
      dv = (an[i] + a) / (b + a);
      a = c / b;
    }
    a = 1.0 / std::sqrt(c * c + 1.0);
    s = (s < 0.0) ? -a : a;
    co = c * s;
  }
  if (m > 1.0) {
    const double t = dv;
    dv = co;
    co = t;
    s = s / d;
  }
  *sn = s;
  *cn = co;
  *dn = dv;
}

double horner(const double* c, int n, double x) {
  double r = 0.0;
  for (int i = n - 1; i >= 0; --i) r = r * x + c[i];
  return r;
}

// `param_is_m`: recursive calls pass the parameter m itself instead of L.
// The top-level `high` reflection flag is applied to the result computed from
// the unreflected argument, as in the reference.
void z_ellipj(zd u, double L, zd* sn, zd* cn, zd* dn, bool top) {
  static const double coeffs[7] = {0.0, 1.0, 2.0, 5.0, 14.0, 42.0, 132.0};
  double m;
  bool high = false;
  if (top) {
    double K[2];
    ellipkkp(L, K);
    high = u.imag() > K[1] / 2.0;
    m = std::exp(-2.0 * kPi * L);
  } else {
    m = L;
  }
  if (m < 4.0 * DBL_EPSILON) {
    const zd si = std::sin(u), co = std::cos(u);
    *sn = si + m / 4.0 * (si * co - u) * co;
    *cn = co + m / 4.0 * (-si * co + u) * si;
    *dn = 1.0 + m / 4.0 * (co * co - si * si - 1.0);
  } else {
    const double kappa = (m > 1e-3) ? (1.0 - std::sqrt(1.0 - m)) / (1.0 + std::sqrt(1.0 - m))
                                    : horner(coeffs, 7, m / 4.0);
    const double mu = kappa * kappa;
    zd s1, c1, d1;
    z_ellipj(u / (1.0 + kappa), mu, &s1, &c1, &d1, false);
    const zd den = 1.0 + kappa * s1 * s1;
    *sn = (1.0 + kappa) * s1 / den;
    *cn = c1 * d1 / den;
    *dn = (1.0 - kappa * s1 * s1) / den;
  }
  if (high) {
    const zd snh = *sn, cnh = *cn, dnh = *dn;
    const zd I(0.0, 1.0);
    *sn = -1.0 / (std::sqrt(m) * snh);
    *cn = I * dnh / (std::sqrt(m) * snh);
    *dn = I * cnh / snh;
  }
}

}  // namespace

extern "C" {

int psfun_gpu_ellipkkp(double L, double* K2) {
  if (!K2) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  ellipkkp(L, K2);
  return PSFUN_SUCCESS;
}

int psfun_gpu_d_ellipj(double u, double L, double* sn, double* cn, double* dn) {
  if (!sn || !cn || !dn) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  sncndn(u, std::exp(-2.0 * kPi * L), sn, cn, dn);
  return PSFUN_SUCCESS;
}

int psfun_gpu_z_ellipj(const double* u, double L, double* sn, double* cn, double* dn) {
  if (!u || !sn || !cn || !dn) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  zd s, c, d;
  z_ellipj(zd(u[0], u[1]), L, &s, &c, &d, true);
  sn[0] = s.real(); sn[1] = s.imag();
  cn[0] = c.real(); cn[1] = c.imag();
  dn[0] = d.real(); dn[1] = d.imag();
  return PSFUN_SUCCESS;
}

double psfun_gpu_horner(const double* coeffs, int n, double x) { return coeffs ? horner(coeffs, n, x) : 0.0; }

int psfun_gpu_hhtmethod1(psfun_zfun zfun, void* ctx, int N, const double* rparams, double* xi, double* c,
                         double* eta, double* sign) {
  if (!zfun || N < 1 || !rparams || !xi || !c || !eta || !sign) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  const double mineig = std::fmin(rparams[0], rparams[1]);
  const double maxeig = std::fmax(rparams[0], rparams[1]);
  if (!(mineig > 0.0) || !(maxeig > mineig)) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  const double q = std::sqrt(maxeig / mineig);
  const double cond = (q - 1.0) / (q + 1.0);
  const double L = -std::log(cond) / kPi;
  double K[2];
  ellipkkp(L, K);
  const double sq = std::sqrt(mineig * maxeig);
  for (int j = 1; j <= N; ++j) {
    const zd t = zd(0.0, 0.5) * K[1] - K[0] + ((2.0 * (j - 1) + 1.0) * K[0]) / N;
    zd u, cn, dn;
    z_ellipj(t, L, &u, &cn, &dn, true);
    const zd x = sq * ((1.0 / cond + u) / (1.0 / cond - u));
    double zin[2] = {x.real(), x.imag()}, zout[2] = {0.0, 0.0};
    zfun(zin, zout, ctx);
    const zd den = 1.0 / cond - u;
    const zd cj = (zd(zout[0], zout[1]) / x) * (cn * dn) / (den * den);
    xi[2 * (j - 1)] = x.real();
    xi[2 * (j - 1) + 1] = x.imag();
    c[2 * (j - 1)] = cj.real();
    c[2 * (j - 1) + 1] = cj.imag();
  }
  *eta = -(4.0 * K[0] * sq) / (cond * kPi * N);
  *sign = -1.0;
  return PSFUN_SUCCESS;
}

// Optimized Talbot contour of Trefethen, Weideman & Schmelzer, "Talbot
// quadratures and rational approximations", BIT 46 (2006) 653-670:
//   z(th) = N (0.5017 th cot(0.6407 th) - 0.6122 + 0.2645 i th),  -pi < th < pi,
// midpoint rule th_k = -pi + (k - 1/2) 2 pi / N, so that
//   exp(M) b ~ sum_k c_k (z_k I - M)^{-1} b,  c_k = exp(z_k) z'(th_k) / (i N).
// For real M and b the nodes th and -th give conjugate terms; this returns the
// N/2 nodes with th > 0 and weights 2 c_k, to be used with the real part.
int psfun_gpu_talbot_rule(int N, double* z, double* c) {
  if (N < 2 || (N & 1) || !z || !c) return PSFUN_ERR_INVALID_ARGS_COMBINATION;
  const double mu = 0.5017, nu = 0.6407, sigma = -0.6122, beta = 0.2645;
  const zd I(0.0, 1.0);
  int j = 0;
  for (int k = 1; k <= N; ++k) {
    const double th = -kPi + (k - 0.5) * 2.0 * kPi / N;
    if (th <= 0.0) continue;
    const double cot = std::cos(nu * th) / std::sin(nu * th);
    const double sn = std::sin(nu * th);
    const zd zk = (double)N * zd(mu * th * cot + sigma, beta * th);
    const zd dz = (double)N * zd(mu * (cot - nu * th / (sn * sn)), beta);
    const zd ck = 2.0 * std::exp(zk) * dz / (I * (double)N);
    z[2 * j] = zk.real();
    z[2 * j + 1] = zk.imag();
    c[2 * j] = ck.real();
    c[2 * j + 1] = ck.imag();
    ++j;
  }
  return PSFUN_SUCCESS;
}

}  // extern "C"
