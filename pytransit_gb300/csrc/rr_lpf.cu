// Sampler parameter vectors to RoadRunner model parameters on the device, as
// BaseLPF.transit_model maps them (pytransit/lpf/lpf.py:435-443): a population
// drawn on the GPU goes to the model (or to the fused log-likelihood) without a
// round trip to the host.
#include <cmath>

#include "rr_device.cuh"
#include "rr_internal.h"

namespace rr {

// G of scipy.constants (CODATA 2018) [m^3 kg^-1 s^-2] and seconds per day, as
// in pytransit/orbits/orbits_py.py:34-42.
constexpr double LPF_G = 6.6743e-11;
constexpr double LPF_D_S = 86400.0;

// pv[ipv, :] = [tc, p, rho, b, k2, (q1, q2) per passband at ld_start, ...]:
//   k = sqrt(k2); t0 = tc - tref; a = as_from_rhop(rho, p)
//   (orbits_py.py:604-618); i = i_from_ba(b, a) = acos(b / a) (orbits_py.py:674-689);
//   (u1, u2) = map_ldc(q1, q2) = (sqrt(q1) 2 q2, sqrt(q1) (1 - 2 q2)) (lpf.py:85-91).
__global__ void lpf_map_kernel(const double* __restrict__ pv, int npv, int ldpv, int npb, int ld_start, double tref,
                               double* __restrict__ k, double* __restrict__ t0, double* __restrict__ p,
                               double* __restrict__ a, double* __restrict__ inc, double* __restrict__ ldc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npv) return;
  const double* v = pv + (size_t)i * ldpv;
  const double period = v[1];
  const double as = pow(LPF_G / (3.0 * PI), 1.0 / 3.0) * pow((period * LPF_D_S) * (period * LPF_D_S) * 1e3 * v[2],
                                                            1.0 / 3.0);
  k[i] = sqrt(v[4]);
  t0[i] = v[0] - tref;
  p[i] = period;
  a[i] = as;
  inc[i] = acos(v[3] / as);
  for (int b = 0; b < npb; ++b) {
    const double q1 = v[ld_start + 2 * b], q2 = v[ld_start + 2 * b + 1];
    const double s = sqrt(q1), t = 2.0 * q2;
    ldc[((size_t)i * npb + b) * 2] = s * t;
    ldc[((size_t)i * npb + b) * 2 + 1] = s * (1.0 - t);
  }
}

}  // namespace rr

using namespace rr;

extern "C" {

int rr_lpf_map(const double* pv, int npv, int ldpv, int npb, int ld_start, double tref, double* k, double* t0,
               double* p, double* a, double* inc, double* ldc, void* stream) {
  if (npv < 0 || npb < 0 || ld_start < 5 || ldpv < ld_start + 2 * npb) return RR_ERR_ARG;
  if (npv == 0) return RR_OK;
  lpf_map_kernel<<<(npv + 127) / 128, 128, 0, as_stream(stream)>>>(pv, npv, ldpv, npb, ld_start, tref, k, t0, p, a,
                                                                    inc, ldc);
  return check_launch("rr_lpf_map");
}

}  // extern "C"
