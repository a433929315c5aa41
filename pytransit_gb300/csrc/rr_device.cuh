// Device-side building blocks of the RoadRunner evaluation path.
//
// FP64 pieces follow the reference's numba kernels operation by operation
// (hpparvi/PyTransit 2.8.1: pytransit/models/roadrunner/common.py,
// model_full.py, pytransit/models/numba/ldmodels.py); FP32 pieces are the
// per-sample arithmetic of the split-precision flux kernel.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <math_constants.h>

namespace rr {

constexpr double PI = 3.141592653589793238462643383279502884;

// ---------------------------------------------------------------------------
// Circle-circle intersection (common.py:6-73)
// ---------------------------------------------------------------------------

// circle_circle_intersection_area, common.py:37-49 (two-arccos form, used for
// the weight tables only).
__device__ inline double cci_acos(double r1, double r2, double b) {
  if (r1 < b - r2) return 0.0;
  if (r1 >= b + r2) return PI * r2 * r2;
  if (b - r2 <= -r1) return PI * r1 * r1;
  return r2 * r2 * acos((b * b + r2 * r2 - r1 * r1) / (2 * b * r2)) +
         r1 * r1 * acos((b * b + r1 * r1 - r2 * r2) / (2 * b * r1)) -
         0.5 * sqrt((-b + r2 + r1) * (b + r2 - r1) * (b - r2 + r1) * (b + r2 + r1));
}

// Descending sort of three lengths (tsort, common.py:6-33).
template <typename R>
__device__ inline void tsort(R r1, R r2, R b, R& x, R& y, R& z) {
  if (r1 > r2) {
    if (r1 > b) { x = r1; if (r2 > b) { y = r2; z = b; } else { y = b; z = r2; } }
    else { x = b; y = r1; z = r2; }
  } else {
    if (r2 > b) { x = r2; if (r1 > b) { y = r1; z = b; } else { y = b; z = r1; } }
    else { x = b; y = r2; z = r1; }
  }
}

// Overlap area of circles of radii r1, r2 at separation b in FP32, by the
// kite form of Agol et al. 2020 (the stable counterpart of cci_acos;
// circle_circle_intersection_area_kite, common.py:53-73, for any r1).
__device__ inline float cci_kite_f32(float r1, float r2, float b) {
  const float pi = 3.14159265358979f;
  if (r1 < b - r2) return 0.0f;
  if (r1 >= b + r2) return pi * r2 * r2;
  if (b - r2 <= -r1) return pi * r1 * r1;
  float x, y, w;
  tsort<float>(r1, r2, b, x, y, w);
  const float ak = 0.5f * sqrtf(fmaxf((x + (y + w)) * (w - (x - y)) * (w + (x - y)) * (x + (y - w)), 0.0f));
  const float k0 = atan2f(2.0f * ak, (r2 - r1) * (r2 + r1) + b * b);
  const float k1 = atan2f(2.0f * ak, (r1 - r2) * (r1 + r2) + b * b);
  return r1 * r1 * k1 + r2 * r2 * k0 - ak;
}

// Area of the overlap of the unit stellar disk and a planet of radius k at
// separation z: circle_circle_intersection_area_kite(1, k, z), common.py:53-73
// (Agol et al. 2020).  kappa0 receives the second return value.
template <typename R>
__device__ inline R ccia_star(R k, R z, R& kappa0) {
  const R one = R(1);
  const R pi = R(PI);
  if (one + k <= z) { kappa0 = R(0); return R(0); }
  if (fabs(one - k) < z && z <= one + k) {
    R x, y, w;
    tsort<R>(one, k, z, x, y, w);
    R a_kite = R(0.5) * sqrt((x + (y + w)) * (w - (x - y)) * (w + (x - y)) * (x + (y - w)));
    R k0 = atan2(R(2) * a_kite, (k - one) * (k + one) + z * z);
    R k1 = atan2(R(2) * a_kite, (one - k) * (one + k) + z * z);
    kappa0 = k0;
    return one * one * k1 + k * k * k0 - a_kite;
  }
  if (z <= one - k) { kappa0 = pi; return pi * k * k; }
  if (z <= k - one) { kappa0 = R(0); return pi; }
  kappa0 = R(CUDART_NAN);
  return R(CUDART_NAN);
}

// The kite branch of ccia_star<float> (|1 - k| < z <= 1 + k) without
// branches: the three lengths sorted by a min/max network (exact), then the
// same expressions in the same order, so the value equals ccia_star<float>'s.
__device__ __forceinline__ float kite_star_f32(float k, float z) {
  const float a = fmaxf(1.0f, k), b = fminf(1.0f, k);
  const float x = fmaxf(a, z), t = fminf(a, z);
  const float y = fmaxf(b, t), w = fminf(b, t);
  const float a_kite = 0.5f * sqrtf((x + (y + w)) * (w - (x - y)) * (w + (x - y)) * (x + (y - w)));
  const float k0 = atan2f(2.0f * a_kite, (k - 1.0f) * (k + 1.0f) + z * z);
  const float k1 = atan2f(2.0f * a_kite, (1.0f - k) * (1.0f + k) + z * z);
  return 1.0f * 1.0f * k1 + k * k * k0 - a_kite;
}

// kite_star_f32 for k <= 1/4 with one arctangent: the star's half-angle
// kappa1 (< pi/2 for k < 1) has sin(kappa1) = h, the half-chord, and the kite
// of diagonals z and 2h has area a_kite = z h, so kappa1 = asin(a_kite / z)
// with h <= k <= 1/4, where the Maclaurin series of arcsine to h^11,
//   asin h = h (1 + h^2/6 + 3h^4/40 + 5h^6/112 + 35h^8/1152 + 63h^10/2816),
// has a remainder below 1e-9 relative (the next term is 231 h^12 / 13312).
__device__ __forceinline__ float kite_star_f32_smallk(float k, float z) {
  const float a = fmaxf(1.0f, k), b = fminf(1.0f, k);
  const float x = fmaxf(a, z), t = fminf(a, z);
  const float y = fmaxf(b, t), w = fminf(b, t);
  const float a_kite = 0.5f * sqrtf((x + (y + w)) * (w - (x - y)) * (w + (x - y)) * (x + (y - w)));
  const float k0 = atan2f(2.0f * a_kite, (k - 1.0f) * (k + 1.0f) + z * z);
  const float h = a_kite / z, h2 = h * h;
  const float k1 = h * fmaf(h2, fmaf(h2, fmaf(h2, fmaf(h2, fmaf(h2, 63.0f / 2816.0f, 35.0f / 1152.0f), 5.0f / 112.0f),
                                                  3.0f / 40.0f), 1.0f / 6.0f), 1.0f);
  return k1 + k * k * k0 - a_kite;
}

// The same area with its partial derivatives: dA/dk = 2 k kappa0 (the
// reference's dfdk, common.py:105-114) and dA/dz = -2 A_kite / z (its dfdb,
// common.py:117-128).
template <typename R>
__device__ inline R ccia_star_grad(R k, R z, R& dadk, R& dadz) {
  const R one = R(1);
  const R pi = R(PI);
  if (one + k <= z) { dadk = R(0); dadz = R(0); return R(0); }
  if (fabs(one - k) < z && z <= one + k) {
    R x, y, w;
    tsort<R>(one, k, z, x, y, w);
    R a_kite = R(0.5) * sqrt((x + (y + w)) * (w - (x - y)) * (w + (x - y)) * (x + (y - w)));
    R k0 = atan2(R(2) * a_kite, (k - one) * (k + one) + z * z);
    R k1 = atan2(R(2) * a_kite, (one - k) * (one + k) + z * z);
    dadk = R(2) * k * k0;
    dadz = -R(2) * a_kite / z;
    return one * one * k1 + k * k * k0 - a_kite;
  }
  if (z <= one - k) { dadk = R(2) * pi * k; dadz = R(0); return pi * k * k; }
  if (z <= k - one) { dadk = R(0); dadz = R(0); return pi; }
  dadk = dadz = R(CUDART_NAN);
  return R(CUDART_NAN);
}

// interpolate_mean_limb_darkening_s, common.py:225-233.  The reference reads
// lda[ng] for g in [1-1e-7, 1]; the index is clamped to ng-2 here.
__device__ inline double interp_ldm_f64(double g, double dg, const double* lda, int ng) {
  if (g < 0.0) return CUDART_NAN;
  if (g > 1.0) return 0.0;
  int i = (int)floor(g / dg);
  if (i > ng - 2) i = ng - 2;
  double a = (g - i * dg) / dg;
  return (1.0 - a) * lda[i] + a * lda[i + 1];
}

// ---------------------------------------------------------------------------
// Limb-darkening laws (pytransit/models/numba/ldmodels.py:23-140)
// ---------------------------------------------------------------------------

enum LdLaw : int {
  LD_UNIFORM = 0, LD_LINEAR = 1, LD_QUADRATIC = 2, LD_QUADRATIC_TRI = 3, LD_NONLINEAR = 4,
  LD_GENERAL = 5, LD_SQUARE_ROOT = 6, LD_LOGARITHMIC = 7, LD_EXPONENTIAL = 8, LD_POWER_2 = 9,
  LD_POWER_2_PM = 10, LD_NLAWS = 11
};

template <typename R>
__device__ inline R ld_value(int law, R mu, const R* pv, int npar) {
  const R one = R(1);
  switch (law) {
    case LD_UNIFORM: return one;
    case LD_LINEAR: return one - pv[0] * (one - mu);
    case LD_QUADRATIC: return one - pv[0] * (one - mu) - pv[1] * (one - mu) * (one - mu);
    case LD_QUADRATIC_TRI: {
      R a = sqrt(pv[0]), b = R(2) * pv[1];
      R u = a * b, v = a * (one - b);
      return one - u * (one - mu) - v * (one - mu) * (one - mu);
    }
    case LD_NONLINEAR:
      return one - pv[0] * (one - sqrt(mu)) - pv[1] * (one - mu) - pv[2] * (one - pow(mu, R(1.5))) -
             pv[3] * (one - mu * mu);
    case LD_GENERAL: {
      R s = R(0);
      for (int i = 0; i < npar; ++i) s += pv[i] * (one - pow(mu, R(i + 1)));
      return s;
    }
    case LD_SQUARE_ROOT: return one - pv[0] * (one - mu) - pv[1] * (one - sqrt(mu));
    case LD_LOGARITHMIC: return one - pv[0] * (one - mu) - pv[1] * mu * log(mu);
    case LD_EXPONENTIAL: return one - pv[0] * (one - mu) - pv[1] / (one - exp(mu));
    case LD_POWER_2: return one - pv[0] * (one - pow(mu, pv[1]));
    case LD_POWER_2_PM: {
      R c = one - pv[0] + pv[1];
      R a = log2(c / pv[1]);
      return one - c * (one - pow(mu, a));
    }
  }
  return R(CUDART_NAN);
}

// Analytic disk integral where the RoadRunner law table has one
// (rrmodel.py:48-58); returns false for laws integrated numerically.
template <typename R>
__device__ inline bool ld_integral(int law, const R* pv, R& istar) {
  const R twopi = R(2.0 * PI);
  switch (law) {
    case LD_UNIFORM: istar = R(PI); return true;
    // ldmodels.py:38-39: 2*pi*1/6*(3-2u) (the reference's normalisation, kept)
    case LD_LINEAR: istar = twopi / R(6) * (R(3) - R(2) * pv[0]); return true;
    case LD_QUADRATIC: istar = twopi / R(12) * (R(-2) * pv[0] - pv[1] + R(6)); return true;
    case LD_QUADRATIC_TRI: {
      R a = sqrt(pv[0]), b = R(2) * pv[1];
      R u = a * b, v = a * (R(1) - b);
      istar = twopi / R(12) * (R(-2) * u - v + R(6));
      return true;
    }
    case LD_POWER_2:
      istar = twopi * (-pv[0] * pv[1] + pv[1] + R(2)) / (R(2) * pv[1] + R(4));
      return true;
  }
  return false;
}

// Derivative of the LD profile I(mu) with respect to coefficient j (for the
// adjoint).  Derived from the laws of ldmodels.py:23-140.
template <typename R>
__device__ inline R ld_dvalue(int law, R mu, const R* pv, int npar, int j) {
  const R one = R(1);
  switch (law) {
    case LD_LINEAR: return -(one - mu);
    case LD_QUADRATIC: return j == 0 ? -(one - mu) : -(one - mu) * (one - mu);
    case LD_QUADRATIC_TRI: {
      R a = sqrt(pv[0]), b = R(2) * pv[1];
      if (j == 0) return -(b / (R(2) * a)) * (one - mu) - ((one - b) / (R(2) * a)) * (one - mu) * (one - mu);
      return -R(2) * a * (one - mu) + R(2) * a * (one - mu) * (one - mu);
    }
    case LD_NONLINEAR:
      switch (j) {
        case 0: return -(one - sqrt(mu));
        case 1: return -(one - mu);
        case 2: return -(one - pow(mu, R(1.5)));
        default: return -(one - mu * mu);
      }
    case LD_GENERAL: return one - pow(mu, R(j + 1));
    case LD_SQUARE_ROOT: return j == 0 ? -(one - mu) : -(one - sqrt(mu));
    case LD_LOGARITHMIC: return j == 0 ? -(one - mu) : -mu * log(mu);
    case LD_EXPONENTIAL: return j == 0 ? -(one - mu) : -one / (one - exp(mu));
    case LD_POWER_2: {
      R ma = pow(mu, pv[1]);
      return j == 0 ? -(one - ma) : pv[0] * ma * log(mu);
    }
    case LD_POWER_2_PM: {
      R c = one - pv[0] + pv[1];
      R a = log2(c / pv[1]);
      R ma = pow(mu, a);
      R dIdc = -(one - ma), dIda = c * ma * log(mu);
      const R il2 = R(1.4426950408889634);  // 1 / ln 2
      if (j == 0) return -dIdc + dIda * (-il2 / c);
      return dIdc + dIda * il2 * (one / c - one / pv[1]);
    }
  }
  return R(0);
}

// Derivative of the analytic disk integral with respect to coefficient j;
// false for laws integrated numerically.
template <typename R>
__device__ inline bool ld_dintegral(int law, const R* pv, int j, R& d) {
  const R twopi = R(2.0 * PI);
  switch (law) {
    case LD_UNIFORM: d = R(0); return true;
    case LD_LINEAR: d = twopi / R(6) * R(-2); return true;
    case LD_QUADRATIC: d = j == 0 ? twopi / R(12) * R(-2) : -twopi / R(12); return true;
    case LD_QUADRATIC_TRI: {
      R a = sqrt(pv[0]), b = R(2) * pv[1];
      if (j == 0) d = twopi / R(12) * (R(-2) * (b / (R(2) * a)) - (R(1) - b) / (R(2) * a));
      else d = twopi / R(12) * (R(-2) * a);
      return true;
    }
    case LD_POWER_2: {
      R N = -pv[0] * pv[1] + pv[1] + R(2), D = R(2) * pv[1] + R(4);
      if (j == 0) d = twopi * (-pv[1]) / D;
      else d = twopi * ((R(1) - pv[0]) * D - R(2) * N) / (D * D);
      return true;
    }
  }
  return false;
}

// ---------------------------------------------------------------------------
// Affine laws.  Every named law except power-2 and power-2-pm is
// I(mu) = sum_b coef_b phi_b(mu) with fixed basis functions phi_b, so the LD
// means reduce to sum_b coef_b (W @ phi_b): per-k-row basis tables replace the
// per-pv matrix-vector products.  basis_count returns 0 for the other laws.
// ---------------------------------------------------------------------------
__host__ __device__ inline int basis_count(int law, int npar) {
  switch (law) {
    case LD_UNIFORM: return 1;
    case LD_LINEAR: return 2;
    case LD_QUADRATIC: case LD_QUADRATIC_TRI: case LD_SQUARE_ROOT: case LD_LOGARITHMIC: case LD_EXPONENTIAL:
      return 3;
    case LD_NONLINEAR: return 5;
    case LD_GENERAL: return npar;
  }
  return 0;
}

__device__ inline double basis_value(int law, int b, double mu) {
  if (law == LD_GENERAL) return 1.0 - pow(mu, (double)(b + 1));
  if (b == 0) return 1.0;
  switch (law) {
    case LD_LINEAR: return -(1.0 - mu);
    case LD_QUADRATIC: case LD_QUADRATIC_TRI: return b == 1 ? -(1.0 - mu) : -(1.0 - mu) * (1.0 - mu);
    case LD_NONLINEAR:
      switch (b) {
        case 1: return -(1.0 - sqrt(mu));
        case 2: return -(1.0 - mu);
        case 3: return -(1.0 - pow(mu, 1.5));
        default: return -(1.0 - mu * mu);
      }
    case LD_SQUARE_ROOT: return b == 1 ? -(1.0 - mu) : -(1.0 - sqrt(mu));
    case LD_LOGARITHMIC: return b == 1 ? -(1.0 - mu) : -mu * log(mu);
    case LD_EXPONENTIAL: return b == 1 ? -(1.0 - mu) : -1.0 / (1.0 - exp(mu));
  }
  return 0.0;
}

// coef[b] of one parameter vector's coefficients pv[npar]
__device__ inline void basis_coefs(int law, const double* pv, int npar, double* coef) {
  switch (law) {
    case LD_GENERAL:
      for (int i = 0; i < npar; ++i) coef[i] = pv[i];
      return;
    case LD_QUADRATIC_TRI: {
      double a = sqrt(pv[0]), b = 2 * pv[1];
      coef[0] = 1.0; coef[1] = a * b; coef[2] = a * (1. - b);
      return;
    }
    default:
      coef[0] = 1.0;
      for (int i = 1; i < basis_count(law, npar); ++i) coef[i] = pv[i - 1];
  }
}

// ---------------------------------------------------------------------------
// Orbit layer: Taylor coefficients of the sky position about conjunction
// ---------------------------------------------------------------------------

// Restatement of meepmeep's solve2d(0, p, a, i, e, w) (called at
// model_full.py:60): exact time derivatives of the Keplerian sky position at
// conjunction (f = pi/2 - w, orbits_py.py:83-86), propagated as a Taylor jet of
// r'' = -mu r/|r|^3.  c[0..4] are the x coefficients, c[5..9] the y ones
// (x(t) = sum c[j] t^j, layout of gdmodel.py:441-442); sky axes as
// taylor_z.py:62-76.
// Eccentric anomaly from the mean anomaly by Newton's method, |err| <= 1e-8
// (ea_newton_s, pytransit/orbits/orbits_py.py:145-154).
__device__ inline double ea_newton(double M, double e) {
  double E = M, err = 0.05;
  for (int k = 0; fabs(err) > 1e-8 && k < 1000; ++k) {
    err = E - e * sin(E) - M;
    E = E - err / (1.0 - e * cos(E));
  }
  return E;
}

// solve2d about t = phase (days from mid-transit; the mid-eclipse for the
// eclipse models): the Keplerian state at that time (mean anomaly from the
// one at conjunction, f = pi/2 - w, plus n phase), then the Taylor jet of
// solve2d_conj below.
__device__ inline void solve2d_phase(double phase, double p, double a, double inc, double e, double w, double* c) {
  const double n = 2.0 * PI / p;
  const double se = sqrt(1.0 - e * e);
  const double f0 = 0.5 * PI - w;
  const double E0 = atan2(se * sin(f0), e + cos(f0));
  const double M = E0 - e * sin(E0) + n * phase;
  const double E = ea_newton(M, e);
  const double f = atan2(se * sin(E) / (1.0 - e * cos(E)), (cos(E) - e) / (1.0 - e * cos(E)));
  const double sf = sin(f), cf = cos(f);
  const double cth = cos(w + f), sth = sin(w + f);
  const double r = a * (1.0 - e * e) / (1.0 + e * cf);
  const double vr = n * a * e * sf / se;
  const double vt = n * a * (1.0 + e * cf) / se;
  double P0x = r * cth, P0y = r * sth;
  double P1x = vr * cth - vt * sth, P1y = vr * sth + vt * cth;
  const double mu = n * n * a * a * a;
  const double alpha = -1.5;
  const double q0 = P0x * P0x + P0y * P0y;
  const double q1 = 2.0 * (P0x * P1x + P0y * P1y);
  const double s0 = 1.0 / (q0 * sqrt(q0));
  const double P2x = -mu * s0 * P0x / 2.0, P2y = -mu * s0 * P0y / 2.0;
  const double s1 = alpha * q1 * s0 / q0;
  const double P3x = -mu * (s0 * P1x + s1 * P0x) / 6.0;
  const double P3y = -mu * (s0 * P1y + s1 * P0y) / 6.0;
  const double q2 = 2.0 * (P0x * P2x + P0y * P2y) + (P1x * P1x + P1y * P1y);
  const double s2 = ((alpha - 1.0) * q1 * s1 + 2.0 * alpha * q2 * s0) / (2.0 * q0);
  const double P4x = -mu * (s0 * P2x + s1 * P1x + s2 * P0x) / 12.0;
  const double P4y = -mu * (s0 * P2y + s1 * P1y + s2 * P0y) / 12.0;
  const double ci = cos(inc);
  c[0] = -P0x; c[1] = -P1x; c[2] = -P2x; c[3] = -P3x; c[4] = -P4x;
  c[5] = -ci * P0y; c[6] = -ci * P1y; c[7] = -ci * P2y; c[8] = -ci * P3y; c[9] = -ci * P4y;
}

__device__ inline void solve2d_conj(double p, double a, double inc, double e, double w, double* c) {
  double n = 2.0 * PI / p;
  double se = sqrt(1.0 - e * e);
  double sf = cos(w), cf = sin(w);  // f = pi/2 - w
  double r = a * (1.0 - e * e) / (1.0 + e * cf);
  double vr = n * a * e * sf / se;
  double vt = n * a * (1.0 + e * cf) / se;
  // in-plane position/velocity with w + f = pi/2
  double P0x = 0.0, P0y = r;
  double P1x = -vt, P1y = vr;
  double mu = n * n * a * a * a;
  const double alpha = -1.5;
  double q0 = P0x * P0x + P0y * P0y;
  double q1 = 2.0 * (P0x * P1x + P0y * P1y);
  double s0 = 1.0 / (q0 * sqrt(q0));
  double P2x = -mu * s0 * P0x / 2.0, P2y = -mu * s0 * P0y / 2.0;
  double s1 = alpha * q1 * s0 / q0;
  double P3x = -mu * (s0 * P1x + s1 * P0x) / 6.0;
  double P3y = -mu * (s0 * P1y + s1 * P0y) / 6.0;
  double q2 = 2.0 * (P0x * P2x + P0y * P2y) + (P1x * P1x + P1y * P1y);
  double s2 = ((alpha - 1.0) * q1 * s1 + 2.0 * alpha * q2 * s0) / (2.0 * q0);
  double P4x = -mu * (s0 * P2x + s1 * P1x + s2 * P0x) / 12.0;
  double P4y = -mu * (s0 * P2y + s1 * P1y + s2 * P0y) / 12.0;
  double ci = cos(inc);
  c[0] = -P0x; c[1] = -P1x; c[2] = -P2x; c[3] = -P3x; c[4] = -P4x;
  c[5] = -ci * P0y; c[6] = -ci * P1y; c[7] = -ci * P2y; c[8] = -ci * P3y; c[9] = -ci * P4y;
}

// solve2d_conj in FP32 for the split path, whose flux kernel reads the
// coefficients as FP32 anyway.  Each coefficient carries a few FP32 roundings
// more than the FP64 jet rounded once (relative error ~1e-7, |dz| ~1e-7 near
// transit), and the FP64 pipe, 1/64 of the FP32 rate on this GPU, drops out
// of the prologue's serial chain.  cos i is taken as sin(pi/2 - i) of the
// small angle pi/2 - i formed in FP64, so that b = a cos i keeps its relative
// precision for near-edge-on orbits with large a; sin w and cos w only enter
// multiplied by e.
__device__ inline void solve2d_conj_f32(double p, double a, double inc, double e, double w, float* c) {
  const float af = (float)a, ef = (float)e;
  const float n = (float)(2.0 * PI) / (float)p;
  const float se = sqrtf(1.0f - ef * ef);
  float sf = 1.0f, cf = 0.0f;   // f = pi/2 - w: sin f = cos w, cos f = sin w
  if (ef != 0.0f) sincosf((float)w, &cf, &sf);
  const float r = af * (1.0f - ef * ef) / (1.0f + ef * cf);
  const float vr = n * af * ef * sf / se;
  const float vt = n * af * (1.0f + ef * cf) / se;
  const float P0x = 0.0f, P0y = r;
  const float P1x = -vt, P1y = vr;
  const float mu = n * n * af * af * af;
  const float alpha = -1.5f;
  const float q0 = P0x * P0x + P0y * P0y;
  const float q1 = 2.0f * (P0x * P1x + P0y * P1y);
  const float s0 = 1.0f / (q0 * sqrtf(q0));
  const float P2x = -mu * s0 * P0x / 2.0f, P2y = -mu * s0 * P0y / 2.0f;
  const float s1 = alpha * q1 * s0 / q0;
  const float P3x = -mu * (s0 * P1x + s1 * P0x) / 6.0f;
  const float P3y = -mu * (s0 * P1y + s1 * P0y) / 6.0f;
  const float q2 = 2.0f * (P0x * P2x + P0y * P2y) + (P1x * P1x + P1y * P1y);
  const float s2 = ((alpha - 1.0f) * q1 * s1 + 2.0f * alpha * q2 * s0) / (2.0f * q0);
  const float P4x = -mu * (s0 * P2x + s1 * P1x + s2 * P0x) / 12.0f;
  const float P4y = -mu * (s0 * P2y + s1 * P1y + s2 * P0y) / 12.0f;
  const float ci = sinf((float)(0.5 * PI - inc));
  c[0] = -P0x; c[1] = -P1x; c[2] = -P2x; c[3] = -P3x; c[4] = -P4x;
  c[5] = -ci * P0y; c[6] = -ci * P1y; c[7] = -ci * P2y; c[8] = -ci * P3y; c[9] = -ci * P4y;
}

__device__ inline double sep_c_f64(double t, const double* c) {
  double x = c[0] + t * (c[1] + t * (c[2] + t * (c[3] + t * c[4])));
  double y = c[5] + t * (c[6] + t * (c[7] + t * (c[8] + t * c[9])));
  return sqrt(x * x + y * y);
}

// Contact time by bisection, as pytransit/orbits/taylor_z.py:299-328: bracket
// [0, s*2/vx], tolerance 1e-6 d, at most 100 steps.
__device__ inline double contact_point(double k, int point, const double* c) {
  double s = (point == 1 || point == 2) ? -1.0 : 1.0;
  double zt = (point == 1 || point == 4) ? 1.0 + k : 1.0 - k;
  double t0 = 0.0;
  double t2 = s * 2.0 / fabs(c[1]);   // the sky speed (dx/dt < 0 about an eclipse)
  double t1 = 0.5 * t2;
  double z0 = sep_c_f64(t0, c) - zt;
  double z1 = sep_c_f64(t1, c) - zt;
  for (int i = 0; fabs(t2 - t0) > 1e-6 && i < 100; ++i) {
    if (z0 * z1 < 0.0) {
      t2 = t1;
      t1 = 0.5 * (t0 + t1);
      z1 = sep_c_f64(t1, c) - zt;
    } else {
      t0 = t1;
      t1 = 0.5 * (t1 + t2);
      z0 = z1;
      z1 = sep_c_f64(t1, c) - zt;
    }
  }
  return t1;
}

// The same bisection on the FP32 coefficients, for the split path: the contact
// times only place the bounding box, which is padded by 0.003 d beyond
// contact, so a ~1e-7 d error in them changes no flux value.
__device__ inline float contact_point_f32(float k, int point, const float* c);

// ---------------------------------------------------------------------------
// Float-float helpers (error-free transformations, Knuth / Dekker)
// ---------------------------------------------------------------------------

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = __fmul_rn(a, b);
  e = __fmaf_rn(a, b, -p);
}

// Exact phase-folded time of one point from its FP32-pair time (hi, lo) and
// the light-curve record (t0 - t_ref pair), starting from the epoch estimate
// n: tc = (hi + lo) - (d0h + d0l) - n (p_hi + p_lo) with error-free
// transformations; n is corrected once if the estimate was one off.
__device__ __forceinline__ float exact_tc_pair(float hi, float lo, float d0h, float d0l, float n, float p_hi,
                                               float p_lo, float& tail) {
  float s1, e1, q1, e2, s2, e3;
  two_sum(hi, -d0h, s1, e1);
  two_prod(n, p_hi, q1, e2);
  two_sum(s1, -q1, s2, e3);
  tail = ((e1 + e3) - e2) + (lo - d0l) - n * p_lo;
  float t = s2 + tail;
  if (t >= 0.5f * p_hi || t < -0.5f * p_hi) {
    n += (t >= 0.5f * p_hi) ? 1.0f : -1.0f;
    two_prod(n, p_hi, q1, e2);
    two_sum(s1, -q1, s2, e3);
    tail = ((e1 + e3) - e2) + (lo - d0l) - n * p_lo;
  }
  return s2;   // tc = s2 + tail
}

__device__ __forceinline__ float exact_tc(float hi, float lo, float d0h, float d0l, float n, float p_hi,
                                          float p_lo) {
  float tail;
  const float s2 = exact_tc_pair(hi, lo, d0h, d0l, n, p_hi, p_lo, tail);
  return s2 + tail;
}

// Horner evaluation of the FP32 Taylor coefficients and the separation.
__device__ __forceinline__ float sep_c_f32(float t, const float* c) {
  float x = fmaf(t, fmaf(t, fmaf(t, fmaf(t, c[4], c[3]), c[2]), c[1]), c[0]);
  float y = fmaf(t, fmaf(t, fmaf(t, fmaf(t, c[9], c[8]), c[7]), c[6]), c[5]);
  return sqrtf(fmaf(x, x, y * y));
}

__device__ inline float contact_point_f32(float k, int point, const float* c) {
  const float s = (point == 1 || point == 2) ? -1.0f : 1.0f;
  const float zt = (point == 1 || point == 4) ? 1.0f + k : 1.0f - k;
  float t0 = 0.0f;
  float t2 = s * 2.0f / fabsf(c[1]);
  float t1 = 0.5f * t2;
  float z0 = sep_c_f32(t0, c) - zt;
  float z1 = sep_c_f32(t1, c) - zt;
  for (int i = 0; fabsf(t2 - t0) > 1e-6f && i < 100; ++i) {
    if (z0 * z1 < 0.0f) {
      t2 = t1;
      t1 = 0.5f * (t0 + t1);
      z1 = sep_c_f32(t1, c) - zt;
    } else {
      t0 = t1;
      t1 = 0.5f * (t1 + t2);
      z0 = z1;
      z1 = sep_c_f32(t1, c) - zt;
    }
  }
  return t1;
}

// Points 1 and 4 of contact_point_f32 (the outer contacts) bisected in one
// loop: each keeps its own bracket and stops on its own test, so the results
// are those of the two separate calls, while the two dependent chains overlap.
__device__ inline void contact_points14_f32(float k, const float* c, float& t1, float& t4) {
  const float zt = 1.0f + k;
  float a0 = 0.0f, a2 = -2.0f / fabsf(c[1]);
  float a1 = 0.5f * a2;
  float b0 = 0.0f, b2 = 2.0f / fabsf(c[1]);
  float b1 = 0.5f * b2;
  const float z00 = sep_c_f32(0.0f, c) - zt;
  float za0 = z00, za1 = sep_c_f32(a1, c) - zt;
  float zb0 = z00, zb1 = sep_c_f32(b1, c) - zt;
  bool ra = true, rb = true;
  for (int i = 0; i < 100; ++i) {
    ra = ra && fabsf(a2 - a0) > 1e-6f;
    rb = rb && fabsf(b2 - b0) > 1e-6f;
    if (!ra && !rb) break;
    if (ra) {
      if (za0 * za1 < 0.0f) {
        a2 = a1;
        a1 = 0.5f * (a0 + a1);
      } else {
        a0 = a1;
        a1 = 0.5f * (a1 + a2);
        za0 = za1;
      }
      za1 = sep_c_f32(a1, c) - zt;
    }
    if (rb) {
      if (zb0 * zb1 < 0.0f) {
        b2 = b1;
        b1 = 0.5f * (b0 + b1);
      } else {
        b0 = b1;
        b1 = 0.5f * (b1 + b2);
        zb0 = zb1;
      }
      zb1 = sep_c_f32(b1, c) - zt;
    }
  }
  t1 = a1;
  t4 = b1;
}

}  // namespace rr
