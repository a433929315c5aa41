// Forward-mode dual numbers with five derivative directions, for the
// derivatives of the orbit's Taylor coefficients with respect to
// (p, a, i, e, w) in the adjoint prologue.
#pragma once
#include <cuda_runtime.h>

namespace rr {

struct D5 {
  double v;
  double d[5];
};

__device__ inline D5 dconst(double v) {
  D5 r;
  r.v = v;
  for (int j = 0; j < 5; ++j) r.d[j] = 0.0;
  return r;
}
__device__ inline D5 dvar(double v, int j) {
  D5 r = dconst(v);
  r.d[j] = 1.0;
  return r;
}
__device__ inline D5 operator+(const D5& a, const D5& b) {
  D5 r; r.v = a.v + b.v;
  for (int j = 0; j < 5; ++j) r.d[j] = a.d[j] + b.d[j];
  return r;
}
__device__ inline D5 operator-(const D5& a, const D5& b) {
  D5 r; r.v = a.v - b.v;
  for (int j = 0; j < 5; ++j) r.d[j] = a.d[j] - b.d[j];
  return r;
}
__device__ inline D5 operator-(const D5& a) {
  D5 r; r.v = -a.v;
  for (int j = 0; j < 5; ++j) r.d[j] = -a.d[j];
  return r;
}
__device__ inline D5 operator*(const D5& a, const D5& b) {
  D5 r; r.v = a.v * b.v;
  for (int j = 0; j < 5; ++j) r.d[j] = a.d[j] * b.v + a.v * b.d[j];
  return r;
}
__device__ inline D5 operator*(double s, const D5& a) {
  D5 r; r.v = s * a.v;
  for (int j = 0; j < 5; ++j) r.d[j] = s * a.d[j];
  return r;
}
__device__ inline D5 operator/(const D5& a, const D5& b) {
  D5 r; r.v = a.v / b.v;
  const double ib = 1.0 / b.v;
  for (int j = 0; j < 5; ++j) r.d[j] = (a.d[j] - r.v * b.d[j]) * ib;
  return r;
}
__device__ inline D5 operator/(const D5& a, double s) {
  D5 r; r.v = a.v / s;
  for (int j = 0; j < 5; ++j) r.d[j] = a.d[j] / s;
  return r;
}
__device__ inline D5 dsqrt(const D5& a) {
  D5 r; r.v = sqrt(a.v);
  const double h = 0.5 / r.v;
  for (int j = 0; j < 5; ++j) r.d[j] = a.d[j] * h;
  return r;
}
__device__ inline D5 dsin(const D5& a) {
  D5 r; r.v = sin(a.v);
  const double c = cos(a.v);
  for (int j = 0; j < 5; ++j) r.d[j] = a.d[j] * c;
  return r;
}
__device__ inline D5 dcos(const D5& a) {
  D5 r; r.v = cos(a.v);
  const double s = -sin(a.v);
  for (int j = 0; j < 5; ++j) r.d[j] = a.d[j] * s;
  return r;
}

// solve2d_conj (rr_device.cuh) on dual numbers: c[0..9] with their
// derivatives with respect to (p, a, i, e, w).
__device__ inline void solve2d_conj_dual(double p_, double a_, double inc_, double e_, double w_, D5* c) {
  const D5 p = dvar(p_, 0), a = dvar(a_, 1), inc = dvar(inc_, 2), e = dvar(e_, 3), w = dvar(w_, 4);
  const D5 one = dconst(1.0);
  const D5 n = dconst(2.0 * 3.141592653589793238462643383279502884) / p;
  const D5 se = dsqrt(one - e * e);
  const D5 sf = dcos(w), cf = dsin(w);
  const D5 r = a * (one - e * e) / (one + e * cf);
  const D5 vr = n * a * e * sf / se;
  const D5 vt = n * a * (one + e * cf) / se;
  const D5 P0x = dconst(0.0), P0y = r;
  const D5 P1x = -vt, P1y = vr;
  const D5 mu = n * n * a * a * a;
  const double alpha = -1.5;
  const D5 q0 = P0x * P0x + P0y * P0y;
  const D5 q1 = 2.0 * (P0x * P1x + P0y * P1y);
  const D5 s0 = one / (q0 * dsqrt(q0));
  const D5 P2x = -(mu * s0 * P0x) / 2.0, P2y = -(mu * s0 * P0y) / 2.0;
  const D5 s1 = alpha * (q1 * s0 / q0);
  const D5 P3x = -(mu * (s0 * P1x + s1 * P0x)) / 6.0;
  const D5 P3y = -(mu * (s0 * P1y + s1 * P0y)) / 6.0;
  const D5 q2 = 2.0 * (P0x * P2x + P0y * P2y) + (P1x * P1x + P1y * P1y);
  const D5 s2 = ((alpha - 1.0) * (q1 * s1) + (2.0 * alpha) * (q2 * s0)) / (2.0 * q0);
  const D5 P4x = -(mu * (s0 * P2x + s1 * P1x + s2 * P0x)) / 12.0;
  const D5 P4y = -(mu * (s0 * P2y + s1 * P1y + s2 * P0y)) / 12.0;
  const D5 ci = dcos(inc);
  c[0] = -P0x; c[1] = -P1x; c[2] = -P2x; c[3] = -P3x; c[4] = -P4x;
  c[5] = -(ci * P0y); c[6] = -(ci * P1y); c[7] = -(ci * P2y); c[8] = -(ci * P3y); c[9] = -(ci * P4y);
}

}  // namespace rr
