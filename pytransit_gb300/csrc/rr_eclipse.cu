// RoadRunner secondary-eclipse models in FP64: the multiplicative eclipse
// model (eclipse_model, pytransit/models/roadrunner/model_eclipse.py:12-81,
// the visible area of the planet disk) and its spectroscopic variant (esmodel,
// model_ecspec.py:13-63, npb flux ratios).  Same orbit layer as the transit
// model, expanded about mid-eclipse, the eclipse time shifted by the light
// travel time across the orbit.
#include <cmath>

#include "rr_device.cuh"
#include "rr_internal.h"

namespace rr {

constexpr int ECL_REC = 16;   // c[0..9], [10] t1, [11] t4, [12] shift, [13] valid, [14] ltt, [15] unused

// Time from mid-transit to mid-eclipse from the mean anomalies at the two
// conjunctions, wrapped to (0, p] (meepmeep's eclipse_time_offset; the
// reference's own eclipse_phase, pytransit/orbits/orbits_py.py:544-555).
__device__ inline double eclipse_time_offset(double p, double e, double w) {
  const double se = sqrt(1.0 - e * e);
  const double etr = atan2(se * sin(0.5 * PI - w), e + cos(0.5 * PI - w));
  const double eec = atan2(se * sin(0.5 * PI + PI - w), e + cos(0.5 * PI + PI - w));
  const double mtr = etr - e * sin(etr), mec = eec - e * sin(eec);
  const double ph = (mec - mtr) * p / (2.0 * PI);
  return ph > 0.0 ? ph : p + ph;
}

// Extra light travel time of the eclipse over the transit in days
// (meepmeep's eclipse_light_travel_time): the line-of-sight distance
// (r_transit + r_eclipse) sin i in stellar radii of rstar solar radii (IAU
// nominal 6.957e8 m) over c.
__device__ inline double eclipse_ltt(double a, double inc, double e, double w, double rstar) {
  const double r_tr = a * (1.0 - e * e) / (1.0 + e * cos(0.5 * PI - w));
  const double r_ec = a * (1.0 - e * e) / (1.0 + e * cos(1.5 * PI - w));
  return (r_tr + r_ec) * sin(inc) * rstar * 6.957e8 / 299792458.0 / 86400.0;
}

// Per pv: validity, eclipse shift, light travel time, Taylor coefficients
// about mid-eclipse and the contact points (model_eclipse.py:38-60).
__global__ void eclipse_prepare_kernel(const double* __restrict__ k, const double* __restrict__ p,
                                       const double* __restrict__ a, const double* __restrict__ inc,
                                       const double* __restrict__ e, const double* __restrict__ w,
                                       const double* __restrict__ rstar, int npv, double* __restrict__ rec) {
  const int pv = blockIdx.x * blockDim.x + threadIdx.x;
  if (pv >= npv) return;
  double* o = rec + (size_t)pv * ECL_REC;
  for (int i = 0; i < ECL_REC; ++i) o[i] = 0.0;
  if (isnan(a[pv]) || a[pv] <= 1.0 || e[pv] < 0.0) return;
  const double shift = eclipse_time_offset(p[pv], e[pv], w[pv]);
  double c[10];
  solve2d_phase(shift, p[pv], a[pv], inc[pv], e[pv], w[pv], c);
  for (int i = 0; i < 10; ++i) o[i] = c[i];
  o[10] = contact_point(k[pv], 1, c);
  o[11] = contact_point(k[pv], 4, c);
  o[12] = shift;
  o[13] = 1.0;
  o[14] = eclipse_ltt(a[pv], inc[pv], e[pv], w[pv], rstar[pv]);
}

// eclipse_model's light curve loop (model_eclipse.py:62-80), one thread per
// (pv, point): pi k^2 outside the padded box, else the mean over the exposure
// samples of the visible area pi k^2 - A(1, k, z).
__global__ void __launch_bounds__(256)
eclipse_flux_kernel(const double* __restrict__ times, int npt, const double* __restrict__ k,
                    const double* __restrict__ t0, int ldt0, const double* __restrict__ p,
                    const int32_t* __restrict__ lcids, const int32_t* __restrict__ epids,
                    const int32_t* __restrict__ nsamples, const double* __restrict__ exptimes,
                    const double* __restrict__ rec, int npv, double* __restrict__ flux, int ldflux) {
  const int pv = blockIdx.z * 65535 + blockIdx.y;
  const int pt = blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= npt || pv >= npv) return;
  const double* o = rec + (size_t)pv * ECL_REC;
  double* out = flux + (size_t)pv * ldflux + pt;
  if (o[13] == 0.0) {
    *out = CUDART_NAN;
    return;
  }
  const int lc = lcids[pt];
  const double kk = k[pv];
  const double pik2 = PI * (kk * kk);
  const double pp = p[pv];
  const double te = __dadd_rn(__dadd_rn(t0[(size_t)pv * ldt0 + epids[lc]], o[12]), o[14]);
  const double t = times[pt];
  const double epoch = floor(__ddiv_rn(__dadd_rn(__dsub_rn(t, te), __dmul_rn(0.5, pp)), pp));
  const double tc = __dsub_rn(t, __dadd_rn(te, __dmul_rn(epoch, pp)));
  const double ex = exptimes[lc];
  const double pad = __dadd_rn(0.003, ex);
  if (!(__dsub_rn(o[10], pad) <= tc && tc <= __dadd_rn(o[11], pad))) {
    *out = pik2;
    return;
  }
  double c[10];
  for (int i = 0; i < 10; ++i) c[i] = o[i];
  const int ns = nsamples[lc];
  double f = 0.0;
  for (int s = 1; s < ns + 1; ++s) {
    const double z = sep_c_f64(tc + ex * ((s - 0.5) / ns - 0.5), c);
    double kap;
    f += pik2 - ccia_star<double>(kk, z, kap);
  }
  *out = f / ns;
}

// esmodel's light curve loop (model_ecspec.py:49-62), one thread per (pv,
// point), all channels: 1 outside the box padded by 0.0015 d + exptime, else
// the mean over the samples of 1 - (f_b A(1, k, z) / pi) / (1 + f_b k^2).
__global__ void __launch_bounds__(256)
es_flux_kernel(const double* __restrict__ times, int npt, const double* __restrict__ k,
               const double* __restrict__ t0, const double* __restrict__ p, const double* __restrict__ fratio,
               int npb, int nsamples0, double exptime0, const double* __restrict__ rec, int npv,
               double* __restrict__ flux, int ldflux) {
  const int pv = blockIdx.z * 65535 + blockIdx.y;
  const int pt = blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= npt || pv >= npv) return;
  const double* o = rec + (size_t)pv * ECL_REC;
  double* out = flux + (size_t)pv * npb * ldflux + pt;
  if (o[13] == 0.0) {
    for (int b = 0; b < npb; ++b) out[(size_t)b * ldflux] = CUDART_NAN;
    return;
  }
  const double kk = k[pv], pp = p[pv];
  const double te = __dadd_rn(__dadd_rn(t0[pv], o[12]), o[14]);
  const double t = times[pt];
  const double epoch = floor(__ddiv_rn(__dadd_rn(__dsub_rn(t, te), __dmul_rn(0.5, pp)), pp));
  const double tc = __dsub_rn(t, __dadd_rn(te, __dmul_rn(epoch, pp)));
  const double pad = __dadd_rn(0.0015, exptime0);
  if (!(__dsub_rn(o[10], pad) <= tc && tc <= __dadd_rn(o[11], pad))) {
    for (int b = 0; b < npb; ++b) out[(size_t)b * ldflux] = 1.0;
    return;
  }
  double c[10];
  for (int i = 0; i < 10; ++i) c[i] = o[i];
  const double* fr = fratio + (size_t)pv * npb;
  for (int b = 0; b < npb; ++b) out[(size_t)b * ldflux] = 0.0;
  for (int s = 1; s < nsamples0 + 1; ++s) {
    const double z = sep_c_f64(tc + exptime0 * ((s - 0.5) / nsamples0 - 0.5), c);
    double kap;
    const double ar = ccia_star<double>(kk, z, kap);
    for (int b = 0; b < npb; ++b)
      out[(size_t)b * ldflux] += 1.0 - (fr[b] * ar / PI) / (1.0 + fr[b] * (kk * kk));
  }
  for (int b = 0; b < npb; ++b) out[(size_t)b * ldflux] /= nsamples0;
}

}  // namespace rr

using namespace rr;

extern "C" {

size_t rr_eclipse_workspace_bytes(int npv) { return sizeof(double) * (size_t)(npv > 0 ? npv : 1) * ECL_REC + 256; }

int rr_eclipse_f64(const double* times, int npt, const double* k, const double* t0, int ldt0, const double* p,
                   const double* a, const double* inc, const double* e, const double* w, const double* rstar,
                   int npv, int nlc, const int32_t* lcids, const int32_t* epids, const int32_t* nsamples,
                   const double* exptimes, void* workspace, size_t workspace_bytes, double* flux, int ldflux,
                   void* stream) {
  if (npt < 0 || npv < 0 || nlc < 1 || ldt0 < 1 || ldflux < npt) return RR_ERR_ARG;
  if (npv == 0 || npt == 0) return RR_OK;
  if (workspace_bytes < rr_eclipse_workspace_bytes(npv)) return RR_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  double* rec = static_cast<double*>(workspace);
  eclipse_prepare_kernel<<<(npv + 63) / 64, 64, 0, s>>>(k, p, a, inc, e, w, rstar, npv, rec);
  dim3 fg((npt + 255) / 256, npv < 65535 ? npv : 65535, (npv + 65534) / 65535);
  eclipse_flux_kernel<<<fg, 256, 0, s>>>(times, npt, k, t0, ldt0, p, lcids, epids, nsamples, exptimes, rec, npv,
                                         flux, ldflux);
  return check_launch("rr_eclipse_f64");
}

int rr_es_f64(const double* times, int npt, const double* k, const double* t0, const double* p, const double* a,
              const double* inc, const double* e, const double* w, const double* rstar, const double* fratio,
              int npv, int npb, int nsamples0, double exptime0, void* workspace, size_t workspace_bytes,
              double* flux, int ldflux, void* stream) {
  if (npt < 0 || npv < 0 || npb < 1 || nsamples0 < 1 || ldflux < npt) return RR_ERR_ARG;
  if (npv == 0 || npt == 0) return RR_OK;
  if (workspace_bytes < rr_eclipse_workspace_bytes(npv)) return RR_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  double* rec = static_cast<double*>(workspace);
  eclipse_prepare_kernel<<<(npv + 63) / 64, 64, 0, s>>>(k, p, a, inc, e, w, rstar, npv, rec);
  dim3 fg((npt + 255) / 256, npv < 65535 ? npv : 65535, (npv + 65534) / 65535);
  es_flux_kernel<<<fg, 256, 0, s>>>(times, npt, k, t0, p, fratio, npb, nsamples0, exptime0, rec, npv, flux, ldflux);
  return check_launch("rr_es_f64");
}

}  // extern "C"
