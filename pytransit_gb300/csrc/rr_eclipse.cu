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
struct EclF64Args {
  const double* times;
  int npt;
  const double *k, *t0;
  int ldt0;
  const double* p;
  const int32_t *lcids, *epids, *nsamples;
  const double *exptimes, *rec;
  int npv;
  double* flux;
  int ldflux;
};

// One point of a valid pv: pi k^2 outside the padded box, else the mean over
// the exposure samples of the visible area pi k^2 - A(1, k, z).  Compiled
// once and called by both flux kernels, so that the compiler's fusing of
// multiplies and adds is the same in both and so are their bits.
__device__ __noinline__ double ecl_point_f64(const EclF64Args& A, int pv, int pt, const double* o) {
  const int lc = A.lcids[pt];
  const double kk = A.k[pv];
  const double pik2 = PI * (kk * kk);
  const double pp = A.p[pv];
  const double te = __dadd_rn(__dadd_rn(A.t0[(size_t)pv * A.ldt0 + A.epids[lc]], o[12]), o[14]);
  const double t = A.times[pt];
  const double epoch = floor(__ddiv_rn(__dadd_rn(__dsub_rn(t, te), __dmul_rn(0.5, pp)), pp));
  const double tc = __dsub_rn(t, __dadd_rn(te, __dmul_rn(epoch, pp)));
  const double ex = A.exptimes[lc];
  const double pad = __dadd_rn(0.003, ex);
  if (!(__dsub_rn(o[10], pad) <= tc && tc <= __dadd_rn(o[11], pad))) return pik2;
  double c[10];
  for (int i = 0; i < 10; ++i) c[i] = o[i];
  const int ns = A.nsamples[lc];
  double f = 0.0;
  for (int s = 1; s < ns + 1; ++s) {
    const double z = sep_c_f64(tc + ex * ((s - 0.5) / ns - 0.5), c);
    double kap;
    f += pik2 - ccia_star<double>(kk, z, kap);
  }
  return f / ns;
}

// eclipse_model's light curve loop (model_eclipse.py:62-80), one thread per
// (pv, point).
__global__ void __launch_bounds__(256) eclipse_flux_kernel(EclF64Args A) {
  const int pv = blockIdx.z * 65535 + blockIdx.y;
  const int pt = blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= A.npt || pv >= A.npv) return;
  const double* o = A.rec + (size_t)pv * ECL_REC;
  A.flux[(size_t)pv * A.ldflux + pt] = o[13] == 0.0 ? CUDART_NAN : ecl_point_f64(A, pv, pt, o);
}

// The same with the fold once per 128-point tile for tiles that reach no box
// (tiles64 from rr_time_tiles_f64).  The fold about the eclipse epoch te is
// non-decreasing in t with the reference's rounding, so a one-light-curve
// tile whose two ends share an epoch and whose two ends' tc miss the padded
// box is pi k^2 at every point: the same bits as eclipse_flux_kernel.  A warp
// tests 32 tiles at once, one per lane.
constexpr int ECL64_WARPS = 4;

__global__ void __launch_bounds__(ECL64_WARPS * 32) eclipse_flux_culled_kernel(EclF64Args A, const double* tiles64) {
  const int pv = blockIdx.z * 65535 + blockIdx.y;
  if (pv >= A.npv) return;   // block-uniform
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = (A.npt + TIME_TILE - 1) / TIME_TILE;
  const int tbase = (blockIdx.x * ECL64_WARPS + warp) * 32;
  if (tbase >= ntiles) return;   // warp-uniform
  const unsigned FULL = 0xffffffffu;
  const double* o = A.rec + (size_t)pv * ECL_REC;
  double* row = A.flux + (size_t)pv * A.ldflux;
  const bool valid = o[13] != 0.0;
  const double kk = A.k[pv];
  const int tile = tbase + lane;
  bool cull = !valid;
  if (valid && tile < ntiles) {
    const double tmin = tiles64[4 * (size_t)tile], tmax = tiles64[4 * (size_t)tile + 1];
    const int lc = (int)tiles64[4 * (size_t)tile + 2];
    if (lc >= 0) {
      const double pp = A.p[pv];
      const double te = __dadd_rn(__dadd_rn(A.t0[(size_t)pv * A.ldt0 + A.epids[lc]], o[12]), o[14]);
      const double e0 = floor(__ddiv_rn(__dadd_rn(__dsub_rn(tmin, te), __dmul_rn(0.5, pp)), pp));
      const double e1 = floor(__ddiv_rn(__dadd_rn(__dsub_rn(tmax, te), __dmul_rn(0.5, pp)), pp));
      if (e0 == e1) {
        const double c = __dadd_rn(te, __dmul_rn(e0, pp));
        const double pad = __dadd_rn(0.003, A.exptimes[lc]);
        cull = __dsub_rn(tmax, c) < __dsub_rn(o[10], pad) || __dsub_rn(tmin, c) > __dadd_rn(o[11], pad);
      }
    }
  }
  const int jn = min(32, ntiles - tbase);
  const unsigned jmask = jn == 32 ? FULL : (1u << jn) - 1u;
  const unsigned cmask = __ballot_sync(FULL, cull) & jmask;
  const double fill = valid ? PI * (kk * kk) : CUDART_NAN;
  for (unsigned m = cmask; m; m &= m - 1u) {
    const int p0 = (tbase + __ffs(m) - 1) * TIME_TILE;
    for (int q = 0; q < 4; ++q)
      if (p0 + 32 * q + lane < A.npt) row[p0 + 32 * q + lane] = fill;
  }
  for (unsigned m = ~cmask & jmask; m; m &= m - 1u) {
    const int p0 = (tbase + __ffs(m) - 1) * TIME_TILE;
    for (int q = 0; q < 4; ++q) {
      const int pt = p0 + 32 * q + lane;
      if (pt < A.npt) row[pt] = ecl_point_f64(A, pv, pt, o);
    }
  }
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

// ---------------------------------------------------------------------------
// Split precision.  The prologue (FP64 eclipse shift, light travel time and
// Taylor jet, one thread per pv) writes an FP32 record per pv and, per light
// curve, the box and the eclipse epoch te - t_ref as an FP32 pair in the
// layout of the transit model's light-curve records (LC_*); the flux kernels
// walk 128-point tiles as the transit flux kernel does: a tile whose time
// range reaches no box copy is a run of stores of the out-of-eclipse value,
// the others fold each point's FP32-pair time exactly (exact_tc) and evaluate
// the samples of the in-box points in FP32.
// ---------------------------------------------------------------------------
constexpr int ECL32 = 16;   // c[0..9], [10] p_hi, [11] p_lo, [12] 1/p_hi, [13] k, [14] flags, [15] pi k^2
constexpr int ECL_NW = 2;   // warps per block of the split flux kernels
constexpr int ECL_CHUNK = 32;

struct EclSplitArgs {
  const float2* times_ff;
  const int32_t* lcids;
  int npt, npv, nlc, npb, ldflux;
  const float *rec, *lcr, *cb;   // [npv][ECL32], [npv][nlc][LC32], ES: [npv][npb] f_b / (pi (1 + f_b k^2))
  float* flux;
};

// The split path's mid-eclipse orbit, for one pv.
//
// The eclipse offset stays FP64, because it is added to t0.  One FP64 sincos
// of w stands in for the four trigonometric calls of eclipse_time_offset
// (sin(pi/2 - w) = cos w and so on), and a circular orbit takes p/2 without
// any.  The light travel time is FP32: it is ~1e-4 d, so its rounding is
// ~1e-11 d.
//
// The jet is about the eclipse conjunction, f = 3 pi/2 - w.  solve2d_phase
// reaches the same Keplerian state by a Newton solve from the mean anomaly at
// mid-transit plus n times the offset.  Here the state is taken in closed
// form, as solve2d_conj_f32 takes the transit's, and it is in FP32:
//   r  = a (1 - e^2) / (1 - e sin w)
//   vr = -n a e cos w / sqrt(1 - e^2)
//   vt = n a (1 - e sin w) / sqrt(1 - e^2)
// with w + f = 3 pi/2, so P0 = (0, -r) and P1 = (vt, -vr).  This agrees with
// the FP64 Newton route to ~2e-15 relative, far below the FP32 rounding of
// the coefficients.
__device__ inline double eclipse_time_offset_split(double p, double e, double w) {
  if (e == 0.0) return 0.5 * p;
  double sw, cw;
  sincos(w, &sw, &cw);
  const double se = sqrt(1.0 - e * e);
  const double etr = atan2(se * cw, e + sw);      // f = pi/2 - w: sin f = cos w, cos f = sin w
  const double eec = atan2(-se * cw, e - sw);     // f = 3 pi/2 - w: sin f = -cos w, cos f = -sin w
  const double mtr = etr - e * sin(etr), mec = eec - e * sin(eec);
  const double ph = (mec - mtr) * p / (2.0 * PI);
  return ph > 0.0 ? ph : p + ph;
}

__device__ inline float eclipse_ltt_f32(float a, float inc_sin, float e, float sw, float rstar) {
  const float r_tr = a * (1.0f - e * e) / (1.0f + e * sw);
  const float r_ec = a * (1.0f - e * e) / (1.0f - e * sw);
  return (r_tr + r_ec) * inc_sin * rstar * (float)(6.957e8 / 299792458.0 / 86400.0);
}

__device__ inline void solve2d_ecl_f32(double p, double a, double inc, double e, float sw, float cw, float* c) {
  const float af = (float)a, ef = (float)e;
  const float n = (float)(2.0 * PI) / (float)p;
  const float se = sqrtf(1.0f - ef * ef);
  const float r = af * (1.0f - ef * ef) / (1.0f - ef * sw);
  const float vr = -n * af * ef * cw / se;
  const float vt = n * af * (1.0f - ef * sw) / se;
  const float P0x = 0.0f, P0y = -r;
  const float P1x = vt, P1y = -vr;
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
  const float ci = sinf((float)(0.5 * PI - inc));   // cos i from the small angle, as solve2d_conj_f32
  c[0] = -P0x; c[1] = -P1x; c[2] = -P2x; c[3] = -P3x; c[4] = -P4x;
  c[5] = -ci * P0y; c[6] = -ci * P1y; c[7] = -ci * P2y; c[8] = -ci * P3y; c[9] = -ci * P4y;
}

// One pv: the FP64 eclipse offset, the FP32 light travel time and jet about
// mid-eclipse (above); contacts by FP32 bisection on the FP32 coefficients
// (they only place the box, padded by pad0 + exptime).  For the spectroscopic model (ES),
// nsamples and exptimes are null and its one record takes ns0 and ex0; the
// channel factors are written too.
__global__ void eclipse_prepare_split_kernel(const double* __restrict__ k, const double* __restrict__ t0, int ldt0,
                                             const double* __restrict__ p, const double* __restrict__ a,
                                             const double* __restrict__ inc, const double* __restrict__ e,
                                             const double* __restrict__ w, const double* __restrict__ rstar,
                                             int npv, int nlc, const int32_t* __restrict__ epids,
                                             const int32_t* __restrict__ nsamples,
                                             const double* __restrict__ exptimes, int ns0, double ex0,
                                             double pad0, double t_ref,
                                             double t_absmax, const double* __restrict__ fratio, int npb,
                                             float* __restrict__ rec, float* __restrict__ lcr,
                                             float* __restrict__ cb) {
  const int pv = blockIdx.x * blockDim.x + threadIdx.x;
  if (pv >= npv) return;
  float* o = rec + (size_t)pv * ECL32;
  const double kk = k[pv], pp = p[pv];
  const bool valid = !(isnan(a[pv]) || a[pv] <= 1.0 || e[pv] < 0.0);
  float cf[10];
  double shift = 0.0, ltt = 0.0;
  float t1 = 0.0f, t4 = 0.0f;
  if (valid) {
    shift = eclipse_time_offset_split(pp, e[pv], w[pv]);
    float sw = 0.0f, cw = 1.0f;
    if (e[pv] != 0.0) sincosf((float)w[pv], &sw, &cw);
    ltt = (double)eclipse_ltt_f32((float)a[pv], sinf((float)inc[pv]), (float)e[pv], sw, (float)rstar[pv]);
    solve2d_ecl_f32(pp, a[pv], inc[pv], e[pv], sw, cw, cf);
    contact_points14_f32((float)kk, cf, t1, t4);
  } else {
    for (int i = 0; i < 10; ++i) cf[i] = 0.0f;
  }
  double d0max = 0.0;
  for (int lc = 0; lc < nlc; ++lc) {
    const double te = t0[(size_t)pv * ldt0 + (epids ? epids[lc] : 0)] + shift + ltt;
    d0max = fmax(d0max, fabs(te - t_ref));
  }
  const float p_hi = __double2float_rn(pp);
  // bound of |fast-test tc - true tc|, as for the transit records
  const double err = ldexp(1.0, -21) * (t_absmax + d0max + pp) + 1e-9;
  int flags = valid ? FLAG_VALID : 0;
  for (int lc = 0; lc < nlc; ++lc) {
    const double ex = exptimes ? exptimes[lc] : ex0;
    const int ns = nsamples ? nsamples[lc] : ns0;
    const double te = t0[(size_t)pv * ldt0 + (epids ? epids[lc] : 0)] + shift + ltt;
    const double d0 = te - t_ref;
    const double pad = pad0 + ex;
    const double lo = (double)t1 - pad, hi = (double)t4 + pad;
    if (hi + 2 * err >= 0.5 * pp || lo - 2 * err <= -0.5 * pp) flags |= FLAG_WIDE;
    float* q = lcr + ((size_t)pv * nlc + lc) * LC32;
    const float d0h = __double2float_rn(d0);
    q[LC_FLO] = (float)(lo - err);
    q[LC_FHI] = (float)(hi + err);
    q[LC_D0H] = d0h;
    q[LC_D0L] = __double2float_rn(d0 - (double)d0h);
    q[LC_LO] = (float)lo;
    q[LC_HI] = (float)hi;
    q[LC_K] = (float)kk;
    q[LC_INV1PK] = 0.0f;
    q[LC_INVIS] = 0.0f;
    q[LC_EXPT] = (float)ex;
    q[LC_INVNS] = 1.0f / (float)ns;
    q[LC_NS] = __int_as_float(ns);
    q[LC_PB] = __int_as_float(0);
    q[13] = q[14] = q[15] = 0.0f;
  }
  for (int i = 0; i < 10; ++i) o[i] = cf[i];
  o[10] = p_hi;
  o[11] = __double2float_rn(pp - (double)p_hi);
  o[12] = 1.0f / p_hi;
  o[13] = (float)kk;
  o[14] = __int_as_float(flags);
  o[15] = (float)(PI * (kk * kk));
  if (cb)
    for (int b = 0; b < npb; ++b) {
      const double f = fratio[(size_t)pv * npb + b];
      cb[(size_t)pv * npb + b] = (float)(f / (PI * (1.0 + f * (kk * kk))));
    }
}

// The in-box value of one point: the mean over its samples of the visible
// planet area pi k^2 - A(1, k, z) (eclipse model) or the mean occulted area
// A(1, k, z) (spectroscopic model, which applies the channel factors after).
// For k <= 1/4 the limb's lens area takes the one-arctangent kite form of the
// transit flux kernel.
template <bool ES>
__device__ __forceinline__ float ecl_point(const float* orb, const float* R, float tc) {
  const float k = orb[13], pik2 = orb[15];
  const int ns = __float_as_int(R[LC_NS]);
  const float ex = R[LC_EXPT], inv_ns = R[LC_INVNS];
  float f = 0.0f;
  for (int s = 0; s < ns; ++s) {
    const float z = sep_c_f32(tc + ex * fmaf((float)s + 0.5f, inv_ns, -0.5f), orb);
    float ar;
    // the kite range of ccia_star (which returns 0 from z = 1 + k on): below
    // the rounded 1 + k, z - 1 < k and the kite's four factors are positive
    if (k <= 0.25f && fabsf(1.0f - k) < z && z < 1.0f + k) {
      ar = kite_star_f32_smallk(k, z);   // a small planet on the limb: one arctangent
    } else {
      float kap;
      ar = ccia_star<float>(k, z, kap);
    }
    f += ES ? ar : pik2 - ar;
  }
  return f * inv_ns;
}

// The flux kernels: blocks of ECL_NW warps, each block a range of at most
// `chunk` consecutive 128-point tiles of one pv, the warps over its tiles.
// Eclipse model: flux[pv, pt] = pi k^2 outside the box, else ecl_point.  ES:
// flux[pv, b, pt] = 1 outside the box, else 1 - cb[pv, b] * mean area.
template <bool ES>
__global__ void __launch_bounds__(ECL_NW * 32) eclipse_flux_split_kernel(EclSplitArgs A, int chunk) {
  __shared__ __align__(16) float orb[ECL32];
  extern __shared__ __align__(16) float ecl_smem[];   // LC records [nlc][LC32], then ES channel factors [npb]
  const int pv = blockIdx.z * 65535 + blockIdx.y;
  if (pv >= A.npv) return;   // block-uniform
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x < ECL32) orb[threadIdx.x] = A.rec[(size_t)pv * ECL32 + threadIdx.x];
  for (int i = threadIdx.x; i < A.nlc * LC32; i += blockDim.x)
    ecl_smem[i] = A.lcr[(size_t)pv * A.nlc * LC32 + i];
  float* cbs = ecl_smem + A.nlc * LC32;
  if (ES)
    for (int i = threadIdx.x; i < A.npb; i += blockDim.x) cbs[i] = A.cb[(size_t)pv * A.npb + i];
  __syncthreads();
  const float* LCR = ecl_smem;
  const int flags = __float_as_int(orb[14]);
  const bool valid = flags & FLAG_VALID, wide = flags & FLAG_WIDE;
  const float p_hi = orb[10], p_lo = orb[11], inv_p = orb[12];
  const float outv = !valid ? __int_as_float(0x7fc00000) : (ES ? 1.0f : orb[15]);
  const int nrow = ES ? A.npb : 1;
  float* fpv = A.flux + (size_t)pv * nrow * A.ldflux;
  const bool vec = ((A.ldflux & 3) == 0) && ((reinterpret_cast<uintptr_t>(A.flux) & 15) == 0);
  const float4 out4 = make_float4(outv, outv, outv, outv);
  const float4* meta = reinterpret_cast<const float4*>(reinterpret_cast<const float*>(A.times_ff) +
                                                       time_meta_offset(A.npt));
  const int ntiles = (A.npt + TIME_TILE - 1) / TIME_TILE;
  const int tb0 = blockIdx.x * chunk, tb1 = min(ntiles, tb0 + chunk);
  // The warp's tiles are tw0 + j ECL_NW, j < ntl, tested 32 at a time (one
  // per lane, as the transit flux kernel does); the culled ones are stored
  // first, walking the set bits of the cull mask, then the others point by
  // point.
  const int tw0 = tb0 + warp;
  const int ntl = tw0 < tb1 ? (tb1 - tw0 + ECL_NW - 1) / ECL_NW : 0;
  const unsigned FULL = 0xffffffffu;
  for (int j0 = 0; j0 < ntl; j0 += 32) {
    bool cull = !valid;
    if (valid && !wide && j0 + lane < ntl) {
      const float4 tm = __ldg(meta + tw0 + (j0 + lane) * ECL_NW);
      const int tlc = ES ? 0 : __float_as_int(tm.z);   // ES: one record for every point
      if (tlc >= 0) {
        const float* R = LCR + tlc * LC32;
        const float smin = tm.x - R[LC_D0H], smax = tm.y - R[LC_D0H];
        const float j0f = ceilf((smin - R[LC_FHI]) * inv_p);
        bool hit = false;
#pragma unroll
        for (int dj = -1; dj <= 1; ++dj) {
          const float jj = j0f + (float)dj;
          hit = hit || (fmaf(jj, p_hi, R[LC_FLO]) <= smax && fmaf(jj, p_hi, R[LC_FHI]) >= smin);
        }
        cull = !hit;
      }
    }
    const int jn = min(32, ntl - j0);
    const unsigned jmask = jn == 32 ? FULL : (1u << jn) - 1u;
    const unsigned cmask = __ballot_sync(FULL, cull) & jmask;
    for (unsigned m = cmask; m; m &= m - 1u) {
      const int p0 = (tw0 + (j0 + __ffs(m) - 1) * ECL_NW) * TIME_TILE;
      const bool full = p0 + TIME_TILE <= A.npt;
      for (int b = 0; b < nrow; ++b) {
        float* row = fpv + (size_t)b * A.ldflux;
        if (vec && full) {
          __stcs(reinterpret_cast<float4*>(row + p0) + lane, out4);
        } else {
          for (int q = 0; q < 4; ++q)
            if (p0 + q * 32 + lane < A.npt) __stcs(row + p0 + q * 32 + lane, outv);
        }
      }
    }
    for (unsigned m = ~cmask & jmask; m; m &= m - 1u) {
      const int tile = tw0 + (j0 + __ffs(m) - 1) * ECL_NW;
      const int p0 = tile * TIME_TILE;
      // slot q of lane l: point p0 + q * 32 + l
      const float4 tm = __ldg(meta + tile);              // min hi, max hi, light curve or -1
      const int tlc = ES ? 0 : __float_as_int(tm.z);     // ES: one record for every point
      float hi[4], lo[4], val[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int pt = p0 + q * 32 + lane;
        const float2 tt = pt < A.npt ? __ldg(A.times_ff + pt) : make_float2(0.0f, 0.0f);
        hi[q] = tt.x;
        lo[q] = tt.y;
        val[q] = ES ? 0.0f : outv;   // ES: the mean area (0 outside the box)
      }
      const float* RT = LCR + (tlc >= 0 ? tlc : 0) * LC32;
      if (!wide && tlc >= 0 && orb[13] <= 0.25f && (tm.y - tm.x) + fmaxf(-RT[LC_LO], RT[LC_HI]) < 0.5f * p_hi) {
        // One light curve, and no point of the tile can fold onto another
        // box copy (span + |box| < p/2): the exact fold once, at the tile's
        // first point, and each point's exact offset from it, as the transit
        // flux kernel does.  The time then takes up to two roundings at its
        // own scale, against one per point below; the area moves with z at
        // most as 2k, so the tile fold is kept to k <= 1/4 (max |dF| 9.7e-8
        // against FP64 on the 8192 x 19,700 workload), and larger planets
        // fold every point.
        const float h0 = __shfl_sync(FULL, hi[0], 0), l0 = __shfl_sync(FULL, lo[0], 0);
        const float n0 = floorf(fmaf(h0 - RT[LC_D0H], inv_p, 0.5f));
        float tail0;
        const float s0 = exact_tc_pair(h0, l0, RT[LC_D0H], RT[LC_D0L], n0, p_hi, p_lo, tail0);
        const float blo = RT[LC_LO], bhi = RT[LC_HI];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float t = (s0 + (hi[q] - h0)) + ((lo[q] - l0) + tail0);
          if (p0 + q * 32 + lane < A.npt && blo <= t && t <= bhi) val[q] = ecl_point<ES>(orb, RT, t);
        }
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int pt = p0 + q * 32 + lane;
          if (pt >= A.npt) continue;
          const float* R = (ES || tlc >= 0) ? RT : LCR + __ldg(A.lcids + pt) * LC32;
          const float sv = hi[q] - R[LC_D0H];
          const float n = floorf(fmaf(sv, inv_p, 0.5f));
          const float r = fmaf(-n, p_hi, sv);
          if (wide || (r >= R[LC_FLO] && r <= R[LC_FHI])) {
            const float t = exact_tc(hi[q], lo[q], R[LC_D0H], R[LC_D0L], n, p_hi, p_lo);
            if (R[LC_LO] <= t && t <= R[LC_HI]) val[q] = ecl_point<ES>(orb, R, t);
          }
        }
      }
      for (int b = 0; b < nrow; ++b) {
        float* row = fpv + (size_t)b * A.ldflux;
        const float c = ES ? cbs[b] : 0.0f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int pt = p0 + q * 32 + lane;
          if (pt < A.npt) __stcs(row + pt, ES ? (valid ? 1.0f - c * val[q] : outv) : val[q]);
        }
      }
    }
  }
}

}  // namespace rr

using namespace rr;

extern "C" {

size_t rr_eclipse_workspace_bytes(int npv) { return sizeof(double) * (size_t)(npv > 0 ? npv : 1) * ECL_REC + 256; }

static int eclipse_f64_launch(const double* times, const double* tiles64, int npt, const double* k, const double* t0,
                              int ldt0, const double* p, const double* a, const double* inc, const double* e,
                              const double* w, const double* rstar, int npv, int nlc, const int32_t* lcids,
                              const int32_t* epids, const int32_t* nsamples, const double* exptimes, void* workspace,
                              size_t workspace_bytes, double* flux, int ldflux, void* stream) {
  if (npt < 0 || npv < 0 || nlc < 1 || ldt0 < 1 || ldflux < npt) return RR_ERR_ARG;
  if (npv == 0 || npt == 0) return RR_OK;
  if (workspace_bytes < rr_eclipse_workspace_bytes(npv)) return RR_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  double* rec = static_cast<double*>(workspace);
  eclipse_prepare_kernel<<<(npv + 63) / 64, 64, 0, s>>>(k, p, a, inc, e, w, rstar, npv, rec);
  EclF64Args A{};
  A.times = times; A.npt = npt; A.k = k; A.t0 = t0; A.ldt0 = ldt0; A.p = p; A.lcids = lcids; A.epids = epids;
  A.nsamples = nsamples; A.exptimes = exptimes; A.rec = rec; A.npv = npv; A.flux = flux; A.ldflux = ldflux;
  if (tiles64) {
    const int ntiles = (npt + TIME_TILE - 1) / TIME_TILE, per = ECL64_WARPS * 32;
    dim3 fg((ntiles + per - 1) / per, npv < 65535 ? npv : 65535, (npv + 65534) / 65535);
    eclipse_flux_culled_kernel<<<fg, ECL64_WARPS * 32, 0, s>>>(A, tiles64);
  } else {
    dim3 fg((npt + 255) / 256, npv < 65535 ? npv : 65535, (npv + 65534) / 65535);
    eclipse_flux_kernel<<<fg, 256, 0, s>>>(A);
  }
  return check_launch("rr_eclipse_f64");
}

int rr_eclipse_f64(const double* times, int npt, const double* k, const double* t0, int ldt0, const double* p,
                   const double* a, const double* inc, const double* e, const double* w, const double* rstar,
                   int npv, int nlc, const int32_t* lcids, const int32_t* epids, const int32_t* nsamples,
                   const double* exptimes, void* workspace, size_t workspace_bytes, double* flux, int ldflux,
                   void* stream) {
  return eclipse_f64_launch(times, nullptr, npt, k, t0, ldt0, p, a, inc, e, w, rstar, npv, nlc, lcids, epids,
                            nsamples, exptimes, workspace, workspace_bytes, flux, ldflux, stream);
}

int rr_eclipse_f64_culled(const double* times, const double* tiles64, int npt, const double* k, const double* t0,
                          int ldt0, const double* p, const double* a, const double* inc, const double* e,
                          const double* w, const double* rstar, int npv, int nlc, const int32_t* lcids,
                          const int32_t* epids, const int32_t* nsamples, const double* exptimes, void* workspace,
                          size_t workspace_bytes, double* flux, int ldflux, void* stream) {
  if (!tiles64) return RR_ERR_ARG;
  return eclipse_f64_launch(times, tiles64, npt, k, t0, ldt0, p, a, inc, e, w, rstar, npv, nlc, lcids, epids,
                            nsamples, exptimes, workspace, workspace_bytes, flux, ldflux, stream);
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

size_t rr_eclipse_split_workspace_bytes(int npv, int nlc, int npb) {
  const size_t n = (size_t)(npv > 0 ? npv : 1);
  return sizeof(float) * n * (ECL32 + (size_t)(nlc > 0 ? nlc : 1) * LC32 + (size_t)(npb > 0 ? npb : 1)) + 3 * 256;
}

static int eclipse_split_launch(bool es, const float* times_ff, double t_ref, double t_absmax, int npt,
                                const double* k, const double* t0, int ldt0, const double* p, const double* a,
                                const double* inc, const double* e, const double* w, const double* rstar,
                                const double* fratio, int npv, int nlc, int npb, const int32_t* lcids,
                                const int32_t* epids, const int32_t* nsamples, const double* exptimes,
                                int ns0, double ex0, double pad0, void* workspace, size_t workspace_bytes, float* flux, int ldflux,
                                void* stream, const char* name) {
  if (workspace_bytes < rr_eclipse_split_workspace_bytes(npv, nlc, npb)) return RR_ERR_WORKSPACE;
  const size_t smem = sizeof(float) * ((size_t)nlc * LC32 + (es ? (size_t)npb : 0));
  if (smem > 48 * 1024) return RR_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  Carve cv(workspace);
  float* rec = cv.take<float>((size_t)npv * ECL32);
  float* lcr = cv.take<float>((size_t)npv * nlc * LC32);
  float* cb = es ? cv.take<float>((size_t)npv * npb) : nullptr;
  // one warp per block: the FP64 chains spread over every SM
  eclipse_prepare_split_kernel<<<(npv + 31) / 32, 32, 0, s>>>(k, t0, ldt0, p, a, inc, e, w, rstar, npv, nlc, epids,
                                                              nsamples, exptimes, ns0, ex0, pad0, t_ref,
                                                              t_absmax, fratio,
                                                              npb, rec, lcr, cb);
  EclSplitArgs A{};
  A.times_ff = reinterpret_cast<const float2*>(times_ff);
  A.lcids = lcids;
  A.npt = npt; A.npv = npv; A.nlc = nlc; A.npb = npb; A.ldflux = ldflux;
  A.rec = rec; A.lcr = lcr; A.cb = cb; A.flux = flux;
  const int ntiles = (npt + TIME_TILE - 1) / TIME_TILE;
  long long chunk = (long long)ntiles * npv / (4LL * sm_count() * ECL_NW * 8);
  chunk = chunk < ECL_NW ? ECL_NW : (chunk > ECL_CHUNK ? ECL_CHUNK : chunk);
  dim3 g((unsigned)((ntiles + chunk - 1) / chunk), npv < 65535 ? npv : 65535, (npv + 65534) / 65535);
  if (es)
    eclipse_flux_split_kernel<true><<<g, ECL_NW * 32, smem, s>>>(A, (int)chunk);
  else
    eclipse_flux_split_kernel<false><<<g, ECL_NW * 32, smem, s>>>(A, (int)chunk);
  return check_launch(name);
}

int rr_eclipse_split(const float* times_ff, double t_ref, double t_absmax, int npt, const double* k,
                     const double* t0, int ldt0, const double* p, const double* a, const double* inc,
                     const double* e, const double* w, const double* rstar, int npv, int nlc, const int32_t* lcids,
                     const int32_t* epids, const int32_t* nsamples, const double* exptimes, void* workspace,
                     size_t workspace_bytes, float* flux, int ldflux, void* stream) {
  if (npt < 0 || npv < 0 || nlc < 1 || ldt0 < 1 || ldflux < npt) return RR_ERR_ARG;
  if (npv == 0 || npt == 0) return RR_OK;
  return eclipse_split_launch(false, times_ff, t_ref, t_absmax, npt, k, t0, ldt0, p, a, inc, e, w, rstar, nullptr,
                              npv, nlc, 1, lcids, epids, nsamples, exptimes, 0, 0.0, 0.003, workspace,
                              workspace_bytes,
                              flux, ldflux, stream, "rr_eclipse_split");
}

int rr_es_split(const float* times_ff, double t_ref, double t_absmax, int npt, const double* k,
                const double* t0, const double* p, const double* a, const double* inc, const double* e,
                const double* w, const double* rstar, const double* fratio, int npv, int npb, int nsamples0,
                double exptime0, void* workspace, size_t workspace_bytes, float* flux, int ldflux, void* stream) {
  if (npt < 0 || npv < 0 || npb < 1 || nsamples0 < 1 || ldflux < npt) return RR_ERR_ARG;
  if (npv == 0 || npt == 0) return RR_OK;
  return eclipse_split_launch(true, times_ff, t_ref, t_absmax, npt, k, t0, 1, p, a, inc, e, w, rstar, fratio, npv,
                              1, npb, nullptr, nullptr, nullptr, nullptr, nsamples0, exptime0, 0.0015, workspace,
                              workspace_bytes, flux, ldflux, stream, "rr_es_split");
}

}  // extern "C"
