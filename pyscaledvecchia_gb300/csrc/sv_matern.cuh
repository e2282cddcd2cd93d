// Matern correlation M_nu(r), its radial factor g(r) = M_nu'(r)/r, and the
// modified Bessel function K_nu used by the general-smoothness form.
//
// Closed forms (nu = 0.5, 1.5, 2.5) follow _covariance.py:49-72 and the
// per-entry code of _covariance.py:111-147; the general form follows
// _matern_general.py:87-116 (M = 2^(1-nu)/Gamma(nu) c^nu K_nu(c),
// c = sqrt(2 nu) r, g via K_{nu-1}, r floored at 1e-7).
//
// K_nu(x) is evaluated with Temme's method (N. M. Temme, "On the numerical
// evaluation of the modified Bessel function of the third kind", J. Comput.
// Phys. 19 (1975) 324-337): write nu = N + mu with |mu| <= 1/2, get K_mu and
// K_{mu+1} from Temme's power series (x <= 1.5) or from Steed's continued
// fraction for the ratio together with Temme's normalising sum (x > 1.5), then
// recur upward K_{a+1} = K_{a-1} + (2a/x) K_a.  The recurrence also yields
// K_{nu-1}, which g needs.  1/Gamma(1 +- mu) come from the Taylor series of
// 1/Gamma(1+z) about 0, whose coefficients were computed for this file to 20
// digits with mpmath (they are the constants of Abramowitz & Stegun 6.1.34
// shifted by one index).
#pragma once
#include <math.h>

#ifndef SV_HD
#define SV_HD __host__ __device__ __forceinline__
#endif

namespace sv {

constexpr double kSqrt3 = 1.7320508075688772;
constexpr double kSqrt5 = 2.23606797749979;
constexpr double kPi = 3.141592653589793;
constexpr double kLn2 = 0.6931471805599453;
constexpr double kRFloor = 1e-7;  // _matern_general.py:87

// Taylor coefficients of 1/Gamma(1+z) about z = 0 (computed to 20 digits
// with mpmath from A&S 6.1.34): 1/Gamma(1+z) = sum_k c_k z^k, |z| <= 1/2
#define SV_RECIP_GAMMA_1P_COEFS \
  1.0, 0.57721566490153286061, -0.65587807152025388108, \
  -0.042002635034095235529, 0.1665386113822914895, -0.042197734555544336748, \
  -0.0096219715278769735621, 0.0072189432466630995424, -0.0011651675918590651121, \
  -0.00021524167411495097282, 0.00012805028238811618615, -0.000020134854780788238656, \
  -1.2504934821426706573e-6, 1.1330272319816958824e-6, -2.0563384169776071035e-7, \
  6.1160951044814158179e-9, 5.0020076444692229301e-9, -1.1812745704870201446e-9, \
  1.0434267116911005105e-10, 7.782263439905071254e-12, -3.6968056186422057082e-12, \
  5.100370287454475979e-13, -2.0583260535665067832e-14, -5.3481225394230179824e-15, \
  1.2267786282382607902e-15, -1.1812593016974587695e-16, 1.1866922547516003326e-18

// 1/Gamma(1+z) by Horner's rule in the coefficients above, |z| <= 1/2
SV_HD double recip_gamma_1p(double z) {
  const double c[27] = {SV_RECIP_GAMMA_1P_COEFS};
  double s = c[26];
  for (int k = 25; k >= 0; --k) s = s * z + c[k];
  return s;
}

// Gamma_1(mu) = (1/Gamma(1-mu) - 1/Gamma(1+mu)) / (2 mu)   (odd part, no cancellation)
// Gamma_2(mu) = (1/Gamma(1-mu) + 1/Gamma(1+mu)) / 2         (even part)
SV_HD void temme_gammas(double mu, double& g1, double& g2, double& rg_plus, double& rg_minus) {
  const double c[27] = {SV_RECIP_GAMMA_1P_COEFS};
  const double m2 = mu * mu;
  // even part: c0 + c2 m^2 + c4 m^4 + ...
  double ev = c[26];
  for (int k = 24; k >= 0; k -= 2) ev = ev * m2 + c[k];
  // odd part / mu: c1 + c3 m^2 + ...
  double od = c[25];
  for (int k = 23; k >= 1; k -= 2) od = od * m2 + c[k];
  g1 = -od;
  g2 = ev;
  rg_plus = ev + mu * od;   // 1/Gamma(1+mu)
  rg_minus = ev - mu * od;  // 1/Gamma(1-mu)
}

// K_mu(x) and K_{mu+1}(x) for |mu| <= 1/2, x > 0 (Temme 1975).
SV_HD void bessel_k_pair(double mu, double x, double& kmu, double& kmu1) {
  const double eps = 1e-17;
  if (x <= 1.5) {
    // Temme's series:  K_mu = sum c_k f_k,  K_{mu+1} = (2/x) sum c_k (p_k - k f_k)
    double g1, g2, rgp, rgm;
    temme_gammas(mu, g1, g2, rgp, rgm);
    const double lnh = -log(0.5 * x);  // ln(2/x)
    const double sig = mu * lnh;
    const double pmu = kPi * mu;
    const double fac = (fabs(pmu) < 1e-15) ? 1.0 : pmu / sin(pmu);
    const double shr = (fabs(sig) < 1e-15) ? 1.0 : sinh(sig) / sig;
    double f = fac * (g1 * cosh(sig) + g2 * shr * lnh);
    const double es = exp(sig);       // (x/2)^(-mu)
    double p = 0.5 * es / rgp;        // (1/2)(x/2)^(-mu) Gamma(1+mu)
    double q = 0.5 / (es * rgm);      // (1/2)(x/2)^(mu) Gamma(1-mu)
    double ck = 1.0;
    const double y = 0.25 * x * x;
    double s0 = f, s1 = p;
    for (int k = 1; k < 500; ++k) {
      const double dk = (double)k;
      f = (dk * f + p + q) / (dk * dk - mu * mu);
      ck *= y / dk;
      p /= (dk - mu);
      q /= (dk + mu);
      const double t0 = ck * f;
      s0 += t0;
      s1 += ck * (p - dk * f);
      if (fabs(t0) < fabs(s0) * eps) break;
    }
    kmu = s0;
    kmu1 = s1 * (2.0 / x);
  } else {
    // Steed's continued fraction for the ratio, with Temme's normalising sum:
    //   K_mu(x) = sqrt(pi/(2x)) e^{-x} / S
    const double a1 = 0.25 - mu * mu;
    double b = 2.0 * (1.0 + x);
    double dd = 1.0 / b;
    double del = dd, h = dd;
    double qm1 = 0.0, qk = 1.0;
    double ak = -a1;
    double cc = a1, qs = a1;
    double S = 1.0 + qs * del;
    for (int i = 2; i < 1000; ++i) {
      ak -= 2.0 * (double)(i - 1);
      cc = -ak * cc / (double)i;
      const double qn = (qm1 - b * qk) / ak;
      qm1 = qk;
      qk = qn;
      qs += cc * qn;
      b += 2.0;
      dd = 1.0 / (b + ak * dd);
      del = (b * dd - 1.0) * del;
      h += del;
      const double ds = qs * del;
      S += ds;
      if (fabs(ds) < fabs(S) * eps) break;
    }
    kmu = sqrt(kPi / (2.0 * x)) * exp(-x) / S;
    kmu1 = kmu * (mu + x + 0.5 - a1 * h) / x;
  }
}

// K_nu(x) and K_{nu-1}(x) for nu >= 0, x > 0.
SV_HD void bessel_k_nu_and_prev(double nu, double x, double& knu, double& knum1) {
  const int N = (int)floor(nu + 0.5);
  const double mu = nu - (double)N;  // in [-1/2, 1/2)
  double k0, k1;                     // K_mu, K_{mu+1}
  bessel_k_pair(mu, x, k0, k1);
  if (N == 0) {
    knu = k0;
    knum1 = k1 - (2.0 * mu / x) * k0;  // K_{mu-1}
    return;
  }
  double km = k0, kc = k1;  // K_{mu+j-1}, K_{mu+j}, j = 1
  for (int j = 1; j < N; ++j) {
    const double kn = km + (2.0 * (mu + (double)j) / x) * kc;
    km = kc;
    kc = kn;
  }
  knu = kc;
  knum1 = km;
}

SV_HD double bessel_k(double nu, double x) {
  double a, b;
  bessel_k_nu_and_prev(fabs(nu), x, a, b);
  return a;
}

// ----------------------------------------------------------------------------
// closed forms: returns M, g (g = M'(r)/r) for nu in {0.5, 1.5, 2.5}
// nu_code: 0 -> 0.5, 1 -> 1.5, 2 -> 2.5
SV_HD void matern_closed(int nu_code, double r, double& M, double& g) {
  if (nu_code == 0) {
    if (r > 0.0) {
      const double e = exp(-r);
      M = e;
      g = -e / r;
    } else {
      M = 1.0;
      g = 0.0;
    }
  } else if (nu_code == 1) {
    const double c = kSqrt3 * r;
    const double e = exp(-c);
    M = (1.0 + c) * e;
    g = -3.0 * e;
  } else {
    // c^2 / 3 as c^2 times 1/3 (a float64 division costs about ten float64
    // instructions; the reference's kernels, compiled with fastmath, may
    // make the same substitution)
    const double c = kSqrt5 * r;
    const double e = exp(-c);
    M = (1.0 + c + c * c * (1.0 / 3.0)) * e;
    g = -(5.0 / 3.0) * (1.0 + c) * e;
  }
}

// general form, _matern_general.py:92-116.  log_coef = (1-nu) ln2 - lgamma(nu).
SV_HD double matern_general_M(double r, double nu, double log_coef) {
  if (r < kRFloor) return 1.0;
  const double c = sqrt(2.0 * nu) * r;
  double knu, knm1;
  bessel_k_nu_and_prev(nu, c, knu, knm1);
  return exp(log_coef + nu * log(c)) * knu;
}

SV_HD void matern_general_Mg(double r, double nu, double log_coef, double& M, double& g) {
  const double rr = r < kRFloor ? kRFloor : r;
  const double s2n = sqrt(2.0 * nu);
  const double c = s2n * rr;
  double knu, knm1;
  bessel_k_nu_and_prev(nu, c, knu, knm1);
  const double pre = exp(log_coef + nu * log(c));
  if (r < kRFloor) {
    M = 1.0;
    g = 0.0;
  } else {
    M = pre * knu;
    g = -(s2n / rr) * pre * knm1;
  }
}

SV_HD double matern_log_coef(double nu) { return (1.0 - nu) * kLn2 - lgamma(nu); }

// ---------------------------------------------------------------------------
// Table of the general-smoothness Matern for a fixed nu (no counterpart in
// the reference, whose _matern_general.py:87-116 calls scipy's kv for every
// entry).  M(c) and G(c) = g(r) = -(2 nu / c) 2^(1-nu)/Gamma(nu) c^nu
// K_{nu-1}(c), c = sqrt(2 nu) r, depend on nu alone: for a fixed nu they are
// interpolated instead of evaluated.  Half-octave intervals [2^e, 2^e sqrt2),
// [2^e sqrt2, 2^(e+1)) of c from 2^elo (elo = floor(log2(sqrt(2 nu) 1e-7)), the
// smallest c the r floor lets through) to 2^9; on each, e^c M(c) and e^c G(c)
// as 16-term Chebyshev series (functions analytic but for c = 0, which lies
// about six half-widths away).  M = e^-c P(t), G = e^-c Q(t), one
// exponential per entry; c >= 2^9 (M < 1e-220) takes the Bessel routine.
// For nu <= 10 the series are within 6e-15 relative of 40-digit values; for
// larger nu, e^c M (close to exp(c - c^2 / (4 nu))) spans too many orders of
// magnitude on an interval (2e-14 at nu = 12.6, 3e-11 at 25.5), so nu > 10
// keeps the per-entry Bessel routine.
// ---------------------------------------------------------------------------
constexpr int kMtabN = 16;       // Chebyshev terms per interval and function
constexpr int kMtabEhi = 9;      // the table covers c < 2^9
constexpr int kMtabEloMin = -40; // smaller nu (c floor below 2^-40): no table
constexpr double kMtabNuMax = 10.0;  // larger nu: no table
constexpr int kMtabMaxDoubles = 2 * (kMtabEhi - kMtabEloMin) * 2 * kMtabN;

// floor(log2(sqrt(2 nu) * 1e-7)): the table's first octave
SV_HD int mtab_elo(double nu) {
  int e = 0;
  frexp(sqrt(2.0 * nu) * kRFloor, &e);
  return e - 1;
}
SV_HD int mtab_intervals(int elo) { return 2 * (kMtabEhi - elo); }

// t in [-1, 1] on the lower ([1, sqrt2)) and upper ([sqrt2, 2)) half of the
// octave, from the mantissa m in [1, 2): t = m S + O
constexpr double kMtabS0 = 4.82842712474619;       // 2 / (sqrt2 - 1)
constexpr double kMtabO0 = -5.82842712474619;      // -(1 + sqrt2) / (sqrt2 - 1)
constexpr double kMtabS1 = 3.414213562373095;      // 2 / (2 - sqrt2)
constexpr double kMtabO1 = -5.82842712474619;      // -(2 + sqrt2) / (2 - sqrt2)
constexpr long long kMtabSqrt2Bits = 0x3FF6A09E667F3BCDLL;  // bits of sqrt(2)

// M(c) and G(c) by the Bessel routine (c > 0)
SV_HD void matern_general_MG_c(double c, double nu, double log_coef, double& M, double& G) {
  double knu, knm1;
  bessel_k_nu_and_prev(nu, c, knu, knm1);
  const double pre = exp(log_coef + nu * log(c));
  M = pre * knu;
  G = -(2.0 * nu / c) * pre * knm1;
}

#ifdef __CUDACC__
// node j of interval iv of the float64 table of nu: e^c M(c) and e^c G(c) at
// the interval's j-th Chebyshev point
__device__ inline void mtab_node(double nu, int elo, int iv, int j, double& fm, double& fg) {
  const int e = elo + iv / 2, half = iv & 1;
  const double tj = cospi((j + 0.5) / kMtabN);
  const double m = half ? (tj - kMtabO1) / kMtabS1 : (tj - kMtabO0) / kMtabS0;
  const double c = ldexp(m, e);
  double knu, knm1;
  bessel_k_nu_and_prev(nu, c, knu, knm1);
  const double sc = exp(c + matern_log_coef(nu) + nu * log(c));  // e^c times the prefactor
  fm = sc * knu;
  fg = -(2.0 * nu / c) * sc * knm1;
}

// Chebyshev coefficient j of an interval of the float64 table from its
// kMtabN node values f
__device__ inline double mtab_coef(const double* f, int j) {
  double a = 0.0;
  for (int i = 0; i < kMtabN; ++i) a = fma(f[i], cospi((double)j * (i + 0.5) / kMtabN), a);
  return a * ((j == 0 ? 1.0 : 2.0) / kMtabN);
}

// interval iv of the float64 table of nu into tab (a CTA of kMtabN threads,
// thread j; fm, fg shared arrays of kMtabN)
__device__ inline void mtab_build_interval(double nu, int iv, double* fm, double* fg, double* tab) {
  const int j = threadIdx.x;
  mtab_node(nu, mtab_elo(nu), iv, j, fm[j], fg[j]);
  __syncthreads();
  tab[(size_t)iv * 2 * kMtabN + j] = mtab_coef(fm, j);
  tab[(size_t)iv * 2 * kMtabN + kMtabN + j] = mtab_coef(fg, j);
}

__device__ __forceinline__ double mtab_clenshaw(const double* cf, double t) {
  const double t2 = t + t;
  double b1 = 0.0, b2 = 0.0;
#pragma unroll
  for (int k = kMtabN - 1; k >= 1; --k) {
    const double b0 = fma(t2, b1, __ldg(cf + k) - b2);
    b2 = b1;
    b1 = b0;
  }
  return fma(t, b1, __ldg(cf) - b2);
}

// M and g = G of matern_general_Mg at r from the table (r floored as
// _matern_general.py:87 does: below 1e-7, M = 1 and g = 0)
__device__ __forceinline__ void matern_table_Mg(const double* tab, int elo, double s2n, double nu,
                                                double log_coef, double r, double& M, double& g,
                                                bool want_g) {
  if (r < kRFloor) {
    M = 1.0;
    g = 0.0;
    return;
  }
  const double c = s2n * r;
  const long long b = __double_as_longlong(c);
  const int e = (int)(b >> 52) - 1023;
  if (e < elo || e >= kMtabEhi) {
    double G;
    matern_general_MG_c(c, nu, log_coef, M, G);
    g = want_g ? G : 0.0;
    return;
  }
  const long long mb = (b & 0x000FFFFFFFFFFFFFLL) | 0x3FF0000000000000LL;
  const double m = __longlong_as_double(mb);
  const int j = mb >= kMtabSqrt2Bits ? 1 : 0;
  const double t = j ? fma(m, kMtabS1, kMtabO1) : fma(m, kMtabS0, kMtabO0);
  const double* cf = tab + (size_t)(2 * (e - elo) + j) * (2 * kMtabN);
  const double ex = exp(-c);
  M = ex * mtab_clenshaw(cf, t);
  g = want_g ? ex * mtab_clenshaw(cf + kMtabN, t) : 0.0;
}

#endif

// nu in {0.5, 1.5, 2.5} -> 0/1/2, else -1
SV_HD int matern_closed_code(double nu) {
  if (nu == 0.5) return 0;
  if (nu == 1.5) return 1;
  if (nu == 2.5) return 2;
  return -1;
}

// ---------------------------------------------------------------------------
// float32 closed forms (the split-precision kernels: likelihood blocks and
// prediction blocks assemble in float32 and factor in float64)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void matern_closed_f32(int code, float r, float& M, float& g) {
  if (code == 0) {
    if (r > 0.0f) {
      const float e = expf(-r);
      M = e;
      g = -e / r;
    } else {
      M = 1.0f;
      g = 0.0f;
    }
  } else if (code == 1) {
    const float c = 1.7320508075688772f * r;
    const float e = expf(-c);
    M = (1.0f + c) * e;
    g = -3.0f * e;
  } else {
    const float c = 2.23606797749979f * r;
    const float e = expf(-c);
    M = (1.0f + c + c * c * (1.0f / 3.0f)) * e;
    g = -(5.0f / 3.0f) * (1.0f + c) * e;
  }
}

// Correlation deficit D = 1 - M(r) with small relative error for every r
// (for nearby points M is close to 1 and 1 - M would lose all of float32's
// digits):  nu = 0.5: -expm1(-r);  for c = sqrt(2 nu) r <= 2,
// nu = 1.5: e^-c c^2 P(c) with P(c) = sum_{k >= 2} c^(k-2) / k!,
// nu = 2.5: e^-c c^2 (P(c) - 1/3)   (1 - M = e^-c (c^2/6 + sum_{k>=3} c^k/k!)),
// P by Horner's rule in c with the constants 1/k!, k = 3 .. 14 (positive
// terms, no cancellation; the terms beyond k = 14 are below 1e-8 of P at
// c = 2).  Measured against 40-digit values on c in [1e-4, 2]: at most 4 ulp,
// 0.8 ulp on average, as the exponential-tail sum it replaces.
__device__ __forceinline__ float matern_deficit_f32(int code, float r) {
  if (code == 0) return -expm1f(-r);
  const float c = (code == 1 ? 1.7320508075688772f : 2.23606797749979f) * r;
  if (c > 2.0f) {
    float M, g;
    matern_closed_f32(code, r, M, g);
    return 1.0f - M;
  }
  constexpr float kInvFact[12] = {1.1470745597729725e-11f, 1.6059043836821613e-10f,
                                  2.08767569878681e-09f,   2.505210838544172e-08f,
                                  2.755731922398589e-07f,  2.7557319223985893e-06f,
                                  2.48015873015873e-05f,   0.0001984126984126984f,
                                  0.001388888888888889f,   0.008333333333333333f,
                                  0.041666666666666664f,   0.16666666666666666f};  // 1/14! .. 1/3!
  float P = kInvFact[0];
#pragma unroll
  for (int t = 1; t < 12; ++t) P = fmaf(P, c, kInvFact[t]);
  P = fmaf(P, c, code == 1 ? 0.5f : 0.16666666666666666f);
  return (expf(-c) * (c * c)) * P;
}

// ---------------------------------------------------------------------------
// float32 table of a fixed general nu (the split kernels; no counterpart in
// the reference, which calls scipy's kv for every entry,
// _matern_general.py:87-116).  On the float64 table's half-octave intervals
// of c = sqrt(2 nu) r, from 2^elo up to 2^6 (for c >= 64, M < 1e-24: D = 1
// and g = 0 in float32), 8-term Chebyshev series with float32 coefficients
//   F(c) = D(c) = 1 - M(c)     on the intervals below 2^esw,
//   F(c) = e^c M(c)            on the others (D = 1 - e^-c F),
//   Q(c) = e^c G(c)            on all of them (g = e^-c Q),
// sixteen floats (four float4) per interval.  2^esw is the first octave at
// or above sqrt(2 max(nu - 1, 1)), where D >= 0.45 for nu <= 50 (D ~ c^2 /
// (4 (nu - 1)) for nu > 1): above it 1 - e^-c F keeps D's relative accuracy.
// Below it, D comes from the series of K_nu through I_-nu and I_nu with the
// leading 1 of M taken out,
//   D(c) = A (c/2)^(2 nu) sum_k x^k / (k! (1+nu)_k) - sum_{k>=1} x^k / (k! (1-nu)_k),
//   x = c^2 / 4,  A = Gamma(1-nu) / Gamma(1+nu) = pi / (sin(pi nu) nu Gamma(nu)^2),
// which keeps D's relative accuracy however small c is (1 - M keeps none of
// it as c -> 0).  Near an integer nu the two sums cancel (the digits lost
// grow as 1 / dist(nu, Z)): the table is built for dist(nu, Z) >= 1e-3 and
// nu <= 8 (at eight terms e^c M and e^c G are within 9e-9 relative up to
// nu = 8.4, 5e-7 at 10.3); other general nu run the float64 kernels.  The
// float64 series is within 1e-13 of 40-digit values below 2^esw for nu from
// 0.3 to 49.7 (at most 52 terms).  Measured in float32 against 40-digit
// values (nu 0.3, 0.8, 1.75, 3.2; c in [2^-20, 64) at the float32 c and t the
// kernels compute): D within 3 ulp and g within 4.2 ulp.
// ---------------------------------------------------------------------------
constexpr int kFtabN = 8;       // Chebyshev terms per interval and function
constexpr int kFtabEhi = 6;     // the float32 table covers c < 2^6
constexpr double kFtabNuMax = 8.0;  // larger nu: no float32 table
constexpr int kFtabIntervals = 2 * (kFtabEhi - kMtabEloMin);
constexpr int kFtabMaxFloats = kFtabIntervals * 2 * kFtabN;  // F and Q
constexpr int kDtabMaxFloats = kFtabIntervals * kFtabN;      // dM/dnu
// one problem's slot in the table region: the float64 tables of nu, nu + h and
// nu - h (the last two for an estimated nu's central difference), the
// float32 table of D and g, and the float32 table of dM/dnu (an estimated nu)
constexpr int kMtabOffP = kMtabMaxDoubles;
constexpr int kMtabOffM = 2 * kMtabMaxDoubles;
constexpr int kFtabOff = 3 * kMtabMaxDoubles;
constexpr int kDtabOff = kFtabOff + kFtabMaxFloats / 2;
constexpr int kMtabSlotDoubles = kDtabOff + kDtabMaxFloats / 2;
static_assert((kFtabOff * 8) % 16 == 0 && (kDtabOff * 8) % 16 == 0 && (kMtabSlotDoubles * 8) % 16 == 0,
              "the float32 tables are read as float4");

// whether a fixed nu gets the float64 table, and the float32 one
SV_HD bool mtab_ok(double nu) {
  return nu > 0.0 && nu <= kMtabNuMax && matern_closed_code(nu) < 0 && mtab_elo(nu) >= kMtabEloMin;
}
SV_HD bool ftab_ok(double nu) {
  return mtab_ok(nu) && nu <= kFtabNuMax && fabs(nu - rint(nu)) >= 1e-3;
}
// an estimated nu of this evaluation: tables of nu and nu +- h (h the
// central difference's step) when all three lie in the table's range
SV_HD bool mtab_est_ok(double nu, double h) {
  return nu - h > 0.0 && nu + h <= kMtabNuMax && mtab_elo(nu - h) >= kMtabEloMin;
}
// an estimated nu of this evaluation in the split forms: float32 tables of
// nu (D, g) and of dM/dnu, whose node values take the series at nu +- h
SV_HD bool ftab_est_ok(double nu, double h) { return ftab_ok(nu) && ftab_ok(nu - h) && ftab_ok(nu + h); }
SV_HD int ftab_intervals(int elo) { return 2 * (kFtabEhi - elo); }
// the first octave whose F is e^c M (at least 1)
SV_HD int ftab_switch(double nu) {
  int e = 0;
  frexp(sqrt(2.0 * fmax(nu - 1.0, 1.0)), &e);
  return e < 1 ? 1 : e;
}

// float32 Matern of a split kernel's block: a closed form, or the table
struct MaternF32 {
  int code;           // 0/1/2: nu = 0.5/1.5/2.5; 3: the float32 table; -1: none
  int elo;            // the table's first octave
  int esw;            // its first octave of F = e^c M
  float s2n;          // sqrt(2 nu)
  const float4* tab;  // four float4 per interval: F, then Q (global or shared)
  const float4* dtab; // estimated nu: two float4 per interval of dM/dnu (or null)
  float nuf;          // nu (the factor of dSigma_nu = s2 nu dM/dnu)
};

#ifdef __CUDACC__
// D(c) for c < 2^esw by the series above (nu at least 1e-3 from an
// integer): terms until both are below 1e-18 of their sums past k = nu + 2
// (at most 52 for nu <= 50), 96 at most
__device__ __forceinline__ double matern_deficit_series(double c, double nu) {
  const double x = 0.25 * c * c;
  const double A = kPi / (sinpi(nu) * nu) * exp(2.0 * nu * log(0.5 * c) - 2.0 * lgamma(nu));
  double s1 = 1.0, t = 1.0, s2 = 0.0, u = 1.0;
  for (int k = 1; k <= 96; ++k) {
    t *= x / (k * (k + nu));
    u *= x / (k * (k - nu));
    s1 += t;
    s2 += u;
    if (k > nu + 2.0 && fabs(t) < 1e-18 * fabs(s1) && fabs(u) < 1e-18 * fabs(s2)) break;
  }
  return A * s1 - s2;
}

// node j of interval iv of the float32 table: F and Q at the interval's
// j-th Chebyshev point
__device__ inline void ftab_node(double nu, int elo, int esw, int iv, int j, double& F,
                                 double& Q) {
  const int e = elo + iv / 2, half = iv & 1;
  const double tj = cospi((j + 0.5) / kFtabN);
  const double m = half ? (tj - kMtabO1) / kMtabS1 : (tj - kMtabO0) / kMtabS0;
  const double c = ldexp(m, e);
  double M, G;
  matern_general_MG_c(c, nu, matern_log_coef(nu), M, G);
  const double ec = exp(c);
  F = e < esw ? matern_deficit_series(c, nu) : ec * M;
  Q = ec * G;
}

// node j of interval iv of the dM/dnu table of an estimated nu: the
// reference's central difference (M(nu + h, r) - M(nu - h, r)) / 2h at
// r = c / sqrt(2 nu) (_matern_general.py:170-176), from the deficits' series
// below 2^esw (M(nu + h) - M(nu - h) = D(nu - h) - D(nu + h), both accurate
// however small) and times e^c from the Bessel routine above
__device__ inline double ftab_dnu_node(double nu, double h, int elo, int esw, int iv, int j) {
  const int e = elo + iv / 2, half = iv & 1;
  const double tj = cospi((j + 0.5) / kFtabN);
  const double m = half ? (tj - kMtabO1) / kMtabS1 : (tj - kMtabO0) / kMtabS0;
  const double c = ldexp(m, e);
  const double r = c / sqrt(2.0 * nu);
  const double nup = nu + h, num = nu - h;
  const double cp = sqrt(2.0 * nup) * r, cmm = sqrt(2.0 * num) * r;
  if (e < esw) return (matern_deficit_series(cmm, num) - matern_deficit_series(cp, nup)) / (2.0 * h);
  double Mp, Mm, G;
  matern_general_MG_c(cp, nup, matern_log_coef(nup), Mp, G);
  matern_general_MG_c(cmm, num, matern_log_coef(num), Mm, G);
  return exp(c) * ((Mp - Mm) / (2.0 * h));
}

// Chebyshev coefficient j of an interval from its kFtabN node values f
__device__ inline float ftab_coef(const double* f, int j) {
  double a = 0.0;
  for (int i = 0; i < kFtabN; ++i) a = fma(f[i], cospi((double)j * (i + 0.5) / kFtabN), a);
  return (float)(a * ((j == 0 ? 1.0 : 2.0) / kFtabN));
}

constexpr float kFtabS0 = 4.82842712474619f;   // t = m S + O, as the float64 table
constexpr float kFtabO0 = -5.82842712474619f;
constexpr float kFtabS1 = 3.414213562373095f;
constexpr float kFtabO1 = -5.82842712474619f;
constexpr int kFtabSqrt2Bits = 0x3FB504F4;     // the smallest float >= sqrt(2)

// interval of c in the float32 table and t in [-1, 1] (a rounding outside
// for c just below 2^elo); -1 for c >= 2^6
__device__ __forceinline__ int ftab_locate(int elo, float c, float& t, int& e) {
  const int bits = __float_as_int(c);
  e = (bits >> 23) - 127;
  if (e >= kFtabEhi) return -1;
  float m;
  int jh = 0;
  if (e < elo) {
    m = c * __int_as_float((127 - elo) << 23);  // c 2^-elo, exact
    e = elo;
  } else {
    const int mb = (bits & 0x007FFFFF) | 0x3F800000;
    m = __int_as_float(mb);
    jh = mb >= kFtabSqrt2Bits ? 1 : 0;
  }
  t = jh ? fmaf(m, kFtabS1, kFtabO1) : fmaf(m, kFtabS0, kFtabO0);
  return 2 * (e - elo) + jh;
}

__device__ __forceinline__ float ftab_clenshaw(float4 lo, float4 hi, float t) {
  const float cf[kFtabN] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
  const float t2 = t + t;
  float b1 = 0.0f, b2 = 0.0f;
#pragma unroll
  for (int k = kFtabN - 1; k >= 1; --k) {
    const float b0 = fmaf(t2, b1, cf[k] - b2);
    b2 = b1;
    b1 = b0;
  }
  return fmaf(t, b1, cf[0] - b2);
}

// D and g of a split kernel's Matern (r floored as _matern_general.py:87
// does: below 1e-7, M = 1 and g = 0)
__device__ __forceinline__ float matern_deficit_f32(const MaternF32& mf, float r) {
  if (mf.code != 3) return matern_deficit_f32(mf.code, r);
  if (r < 1e-7f) return 0.0f;
  const float c = mf.s2n * r;
  float t;
  int e;
  const int iv = ftab_locate(mf.elo, c, t, e);
  if (iv < 0) return 1.0f;
  const float4* p = mf.tab + 4 * iv;
  const float F = ftab_clenshaw(p[0], p[1], t);
  return e < mf.esw ? F : 1.0f - expf(-c) * F;
}

// dM/dnu of an estimated nu (mf.dtab set; r floored as above: 0 below 1e-7)
__device__ __forceinline__ float matern_dnu_f32(const MaternF32& mf, float r) {
  if (r < 1e-7f) return 0.0f;
  const float c = mf.s2n * r;
  float t;
  int e;
  const int iv = ftab_locate(mf.elo, c, t, e);
  if (iv < 0) return 0.0f;
  const float4* p = mf.dtab + 2 * iv;
  const float F = ftab_clenshaw(p[0], p[1], t);
  return e < mf.esw ? F : expf(-c) * F;
}

__device__ __forceinline__ float matern_g_f32(const MaternF32& mf, float r) {
  if (mf.code != 3) {
    float M, g;
    matern_closed_f32(mf.code, r, M, g);
    return g;
  }
  if (r < 1e-7f) return 0.0f;
  const float c = mf.s2n * r;
  float t;
  int e;
  const int iv = ftab_locate(mf.elo, c, t, e);
  if (iv < 0) return 0.0f;
  const float4* p = mf.tab + 4 * iv + 2;
  return expf(-c) * ftab_clenshaw(p[0], p[1], t);
}
#endif

}  // namespace sv
