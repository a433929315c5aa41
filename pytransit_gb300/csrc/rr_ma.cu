// The Mandel & Agol (2002) quadratic limb-darkening model in FP64, the
// independent cross-check of the RoadRunner path: the flux at given centre
// distances (eval_quad_z_s, pytransit/models/numba/ma_quadratic_nb.py:277-389)
// and the full model on the RoadRunner orbit layer (the per-sample flux of
// quadratic_model_v, ma_quadratic_nb.py:532-597, on the same phase fold,
// Taylor-series z and bounding box as rr_flux_f64), so that the two models
// can be compared point by point at any scale.
#include <cmath>

#include "rr_device.cuh"
#include "rr_internal.h"

namespace rr {

// K(k), Abramowitz & Stegun 17.3.34 in m1 = 1 - k^2 (ellk, ma_quadratic_nb.py:110-126).
__device__ inline double ma_ellk(double k) {
  const double m1 = 1.0 - k * k;
  const double ek1 = 1.386294361120 + m1 * (0.096663442590 + m1 * (0.035900923830 + m1 * (0.037425637130 +
                     m1 * 0.014511962120)));
  const double ek2 = (0.50 + m1 * (0.124985935970 + m1 * (0.068802485760 + m1 * (0.033283553460 +
                     m1 * 0.004417870120)))) * log(m1);
  return ek1 - ek2;
}

// E(k), Abramowitz & Stegun 17.3.36 (ellec, ma_quadratic_nb.py:93-107).
__device__ inline double ma_ellec(double k) {
  const double m1 = 1.0 - k * k;
  const double ee1 = 1.0 + m1 * (0.443251414630 + m1 * (0.062606012200 + m1 * (0.047573835460 +
                     m1 * 0.017365064510)));
  const double ee2 = m1 * (0.249983683100 + m1 * (0.092001800370 + m1 * (0.040696975260 +
                     m1 * 0.005264496390))) * log(1.0 / m1);
  return ee1 + ee2;
}

// Pi(n, k) by Bulirsch's (1965) iteration (ellpicb, ma_quadratic_nb.py:55-90);
// 0 when it has not converged after 1000 steps.
__device__ inline double ma_ellpicb(double n, double k) {
  double kc = sqrt(1.0 - k * k), e = kc, p = sqrt(n + 1.0), m0 = 1.0, c = 1.0, d = 1.0 / p;
  for (int it = 0; it < 1000; ++it) {
    const double f = c;
    c = d / p + c;
    double g = e / p;
    d = 2.0 * (f * g + d);
    p = g + p;
    g = m0;
    m0 = kc + m0;
    if (fabs(1.0 - kc / g) > 1e-8) {
      kc = 2.0 * sqrt(e);
      e = kc * m0;
    } else {
      return 0.5 * PI * (c * m0 + d) / (m0 * (m0 + p));
    }
  }
  return 0.0;
}

// Flux at centre distance z for radius ratio k and quadratic coefficients
// (u1, u2), with the reference's case structure and conventions: k within
// 1e-4 of 1/2 becomes 1/2, z within 1e-6 of k moves by +1e-6, z > 1 + k or a
// negative-signed z gives 1, full occultation 0; the limb angles kap0, kap1
// exist only in the ingress/egress branch of the uniform term and are 0 where
// a later branch reads them without it (z = 1 - k exactly), as in the
// reference's compiled code.
__device__ double ma_quad_z(double z, double k, double u1, double u2) {
  const double inv_pi = 1.0 / PI;
  if (fabs(k - 0.5) < 1.0e-4) k = 0.5;
  const double k2 = k * k;
  const double omega = 1.0 - u1 / 3.0 - u2 / 6.0;
  if (fabs(z - k) < 1e-6) z += 1e-6;
  if (z > 1.0 + k || signbit(z)) return 1.0;
  if (k >= 1.0 && z <= k - 1.0) return 0.0;
  const double z2 = z * z, x1 = (k - z) * (k - z), x2 = (k + z) * (k + z), x3 = k * k - z * z;
  double le = 0.0, ld = 0.0, ed = 0.0, kap0 = 0.0, kap1 = 0.0;
  if (z <= 1.0 - k) {
    le = k2;
  } else if (z >= fabs(1.0 - k) && z <= 1.0 + k) {
    kap1 = acos(fmin((1.0 - k2 + z2) / (2.0 * z), 1.0));
    kap0 = acos(fmin((k2 + z2 - 1.0) / (2.0 * k * z), 1.0));
    le = k2 * kap0 + kap1;
    le = (le - 0.5 * sqrt(fmax(4.0 * z2 - (1.0 + z2 - k2) * (1.0 + z2 - k2), 0.0))) * inv_pi;
  }
  const bool edge_at_origin = fabs(z - k) < 1.e-4 * (z + k);
  const bool full_transit = k <= 1.0 && z < (1.0 - k);
  if (edge_at_origin) {
    if (k == 0.5) {
      ld = 1.0 / 3.0 - 4.0 * inv_pi / 9.0;
      ed = 3.0 / 32.0;
    } else if (z > 0.5) {
      const double q = 0.5 / k, Kk = ma_ellk(q), Ek = ma_ellec(q);
      ld = 1.0 / 3.0 + 16.0 * k / 9.0 * inv_pi * (2.0 * k2 - 1.0) * Ek -
           (32.0 * k2 * k2 - 20.0 * k2 + 3.0) / 9.0 * inv_pi / k * Kk;
      ed = 0.5 * inv_pi *
           (kap1 + k2 * (k2 + 2.0 * z2) * kap0 - (1.0 + 5.0 * k2 + z2) / 4.0 * sqrt((1.0 - x1) * (x2 - 1.0)));
    } else if (z < 0.5) {
      const double q = 2.0 * k, Kk = ma_ellk(q), Ek = ma_ellec(q);
      ld = 1.0 / 3.0 + 2.0 / 9.0 * inv_pi * (4.0 * (2.0 * k2 - 1.0) * Ek + (1.0 - 4.0 * k2) * Kk);
      ed = k2 / 2.0 * (k2 + 2.0 * z2);
    }
  } else if (full_transit) {
    const double q = sqrt((x2 - x1) / (1.0 - x1)), Kk = ma_ellk(q), Ek = ma_ellec(q);
    const double Pk = ma_ellpicb(x2 / x1 - 1.0, q);
    ld = 2.0 / 9.0 * inv_pi / sqrt(1.0 - x1) *
         ((1.0 - 5.0 * z2 + k2 + x3 * x3) * Kk + (1.0 - x1) * (z2 + 7.0 * k2 - 4.0) * Ek - 3.0 * x3 / x1 * Pk);
    if (z < k) ld = ld + 2.0 / 3.0;
    if (fabs(k + z - 1.0) < 1.e-4)
      ld = 2.0 / 3.0 * inv_pi * acos(1.0 - 2.0 * k) -
           4.0 / 9.0 * inv_pi * sqrt(k * (1.0 - k)) * (3.0 + 2.0 * k - 8.0 * k2);
    ed = k2 / 2.0 * (k2 + 2.0 * z2);
  } else {
    const double q = sqrt((1.0 - (k - z) * (k - z)) / 4.0 / z / k), Kk = ma_ellk(q), Ek = ma_ellec(q);
    const double Pk = ma_ellpicb(1.0 / x1 - 1.0, q);
    ld = 1.0 / 9.0 * inv_pi / sqrt(k * z) *
         (((1.0 - x2) * (2.0 * x2 + x1 - 3.0) - 3.0 * x3 * (x2 - 2.0)) * Kk +
          4.0 * k * z * (z2 + 7.0 * k2 - 4.0) * Ek - 3.0 * x3 / x1 * Pk);
    if (z < k) ld = ld + 2.0 / 3.0;
    ed = 0.5 * inv_pi *
         (kap1 + k2 * (k2 + 2.0 * z2) * kap0 - (1.0 + 5.0 * k2 + z2) / 4.0 * sqrt((1.0 - x1) * (x2 - 1.0)));
  }
  return 1.0 - ((1.0 - u1 - 2.0 * u2) * le + (u1 + 2.0 * u2) * ld + u2 * ed) / omega;
}

__global__ void ma_quad_z_kernel(const double* __restrict__ z, int n, double k, double u1, double u2,
                                 double* __restrict__ flux) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flux[i] = ma_quad_z(z[i], k, u1, u2);
}

struct MaFluxArgs {
  const double* times;
  const double *k, *t0, *p, *exptimes, *ldc, *orb64;
  const int32_t *lcids, *pbids, *epids, *nsamples;
  int npt, npv, nkc, ldt0, npb, ldflux;
  double* flux;
};

// One thread per (pv, point): the fold, box and samples of flux_f64_kernel,
// the Mandel & Agol flux per sample.
__global__ void __launch_bounds__(256) ma_flux_kernel(MaFluxArgs A) {
  const int pv = blockIdx.z * 65535 + blockIdx.y;
  const int pt = blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= A.npt || pv >= A.npv) return;
  const double* o = A.orb64 + (size_t)pv * ORB64;
  double* out = A.flux + (size_t)pv * A.ldflux + pt;
  if (o[12] == 0.0) {
    *out = CUDART_NAN;
    return;
  }
  const int lc = A.lcids[pt];
  const int pb = A.pbids[lc];
  const int ep = A.epids[lc];
  const double t = A.times[pt];
  const double t0 = A.t0[(size_t)pv * A.ldt0 + ep];
  const double p = A.p[pv];
  const double epoch = floor(__ddiv_rn(__dadd_rn(__dsub_rn(t, t0), __dmul_rn(0.5, p)), p));
  const double tc = __dsub_rn(t, __dadd_rn(t0, __dmul_rn(epoch, p)));
  const double ex = A.exptimes[lc];
  const double pad = __dadd_rn(0.003, ex);
  const double lo = __dsub_rn(o[10], pad), hi = __dadd_rn(o[11], pad);
  if (!(lo <= tc && tc <= hi)) {
    *out = 1.0;
    return;
  }
  const double kk = A.k[(size_t)pv * A.nkc + (A.nkc == A.npb ? pb : 0)];
  const double u1 = A.ldc[((size_t)pv * A.npb + pb) * 2], u2 = A.ldc[((size_t)pv * A.npb + pb) * 2 + 1];
  const int ns = A.nsamples[lc];
  double c[10];
  for (int i = 0; i < 10; ++i) c[i] = o[i];
  double f = 0.0;
  for (int s = 1; s < ns + 1; ++s) {
    const double toff = ex * ((s - 0.5) / ns - 0.5);
    const double z = sep_c_f64(tc + toff, c);
    f += (z > 1.0 + kk) ? 1.0 : ma_quad_z(z, kk, u1, u2);
  }
  *out = f / ns;
}

}  // namespace rr

using namespace rr;

extern "C" {

int rr_ma_quad_z_f64(const double* z, int n, double k, double u1, double u2, double* flux, void* stream) {
  if (n < 0) return RR_ERR_ARG;
  if (n == 0) return RR_OK;
  ma_quad_z_kernel<<<(n + 255) / 256, 256, 0, as_stream(stream)>>>(z, n, k, u1, u2, flux);
  return check_launch("rr_ma_quad_z_f64");
}

int rr_ma_quad_flux_f64(const double* times, int npt, const double* k, int nkc, const double* t0, int ldt0,
                        const double* p, int npv, int nlc, int npb, const int32_t* lcids, const int32_t* pbids,
                        const int32_t* epids, const int32_t* nsamples, const double* exptimes, const double* ldc,
                        const void* workspace, double* flux, int ldflux, void* stream) {
  if (nkc > 1 && nkc != npb) return RR_ERR_SHAPE;
  if (npt < 0 || npv < 0 || nlc < 1 || npb < 1 || nkc < 1 || ldflux < npt) return RR_ERR_ARG;
  if (npv == 0 || npt == 0) return RR_OK;
  MaFluxArgs fa{};
  fa.times = times; fa.k = k; fa.t0 = t0; fa.p = p; fa.exptimes = exptimes; fa.ldc = ldc;
  fa.orb64 = static_cast<const double*>(workspace);   // the first piece of the rr_prepare_f64 workspace
  fa.lcids = lcids; fa.pbids = pbids; fa.epids = epids; fa.nsamples = nsamples;
  fa.npt = npt; fa.npv = npv; fa.nkc = nkc; fa.ldt0 = ldt0; fa.npb = npb; fa.ldflux = ldflux; fa.flux = flux;
  dim3 fg((npt + 255) / 256, npv < 65535 ? npv : 65535, (npv + 65534) / 65535);
  ma_flux_kernel<<<fg, 256, 0, as_stream(stream)>>>(fa);
  return check_launch("rr_ma_quad_flux_f64");
}

}  // extern "C"
