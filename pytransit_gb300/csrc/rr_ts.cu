// Transmission-spectroscopy RoadRunner model (TSModel): npb wavelength
// channels with their own radius ratios share one orbit; LD means at the mean
// radius ratio; the area to first order in k (tsmodel_serial,
// pytransit/models/roadrunner/model_trspec.py:12-93; TransmissionSpectroscopyModel.evaluate,
// pytransit/models/roadrunner/tsmodel.py:46-130).
//
// Semantics kept from the serial reference: only nsamples[0] and exptimes[0]
// are used, one zero epoch t0[pv], a bounding box at the mean radius ratio
// padded by 0.0015 d + exptime, NaN rows for a NaN/<= 1 or e < 0 (no LD
// check), and with a weight table the 3D-table rule kmin <= kmean <= max(k_pv)
// (model_trspec.py:42,48, where max(k) shadows kmax); without one the 2D
// table at kmean.  Output flux[npv, npb, npt].
//
// Three launches: the per-pv prologue (channel records, mean and largest k,
// orbit, box), the LD means (the 2D table rows at kmean reduced against every
// channel's profile), and the flux (rr_ts.cuh: one 128-point tile of one pv
// per unit).  rr_ts_prepare_split / rr_ts_flux_split expose the first two and
// the last separately, so that the serving loop can run the prologue at
// admission and the flux inside its persistent kernel.
#include <cmath>

#include "rr_ts.cuh"

namespace rr {

// Per-pv prologue, one block per pv.  Warp 3 (lane 0) computes the Taylor
// coefficients, which do not depend on k, while warps 0-2 reduce the radius
// ratios to their mean and maximum; then the channel records (threads over
// channels) and the contact points at kmean: the split path bisects both in
// one FP32 loop (its coefficients are FP32, as the RR split prologue's), the
// plain path bisects t1 and t4 in FP64 on two warps at once.
constexpr int TS_PREP_THREADS = 128;
template <typename R, bool SPLIT>
__global__ void __launch_bounds__(TS_PREP_THREADS)
ts_prepare_kernel(const double* __restrict__ k, const double* __restrict__ t0, const double* __restrict__ p,
                  const double* __restrict__ a, const double* __restrict__ inc, const double* __restrict__ e,
                  const double* __restrict__ w, const R* __restrict__ istar, int npv, int npb, double exptime0,
                  double t_ref, double t_absmax, R* __restrict__ orb, R* __restrict__ ch,
                  double* __restrict__ kstat) {
  __shared__ double s_sum[3], s_max[3];
  __shared__ double s_c64[10];
  __shared__ float s_c32[10];
  __shared__ double s_t[2];
  const int pv = blockIdx.x, tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const unsigned FULL = 0xffffffffu;
  const double* kp = k + (size_t)pv * npb;
  const double av = a[pv], ev = e[pv], pp = p[pv];
  const bool valid = !(isnan(av) || av <= 1.0 || ev < 0.0);
  if (warp == 3) {
    if (lane == 0 && valid) {
      if (SPLIT)
        solve2d_conj_f32(pp, av, inc[pv], ev, w[pv], s_c32);
      else
        solve2d_conj(pp, av, inc[pv], ev, w[pv], s_c64);
    }
  } else {
    double sm = 0.0, mx = -INFINITY;
    for (int b = tid; b < npb; b += 96) {
      const double kb = kp[b];
      sm += kb;
      mx = fmax(mx, kb);
    }
    for (int o = 16; o > 0; o >>= 1) {
      sm += __shfl_xor_sync(FULL, sm, o);
      mx = fmax(mx, __shfl_xor_sync(FULL, mx, o));
    }
    if (lane == 0) {
      s_sum[warp] = sm;
      s_max[warp] = mx;
    }
  }
  __syncthreads();
  const double km = ((s_sum[0] + s_sum[1]) + s_sum[2]) / npb;
  const double kx = fmax(fmax(s_max[0], s_max[1]), s_max[2]);
  for (int b = tid; b < npb; b += TS_PREP_THREADS) {
    R* c = ch + ((size_t)pv * npb + b) * TS_CH;
    const double kb = kp[b];
    c[0] = (R)(kb * kb / (km * km));
    c[1] = (R)(kb - km);
    const R is = istar[(size_t)pv * npb + b];
    c[2] = isfinite((double)is) ? R(1) / is : R(CUDART_NAN);
    c[3] = R(0);
  }
  const double pad = 0.0015 + exptime0;
  if (valid) {
    if (SPLIT) {
      if (tid == 0) {
        float t1, t4;
        contact_points14_f32((float)km, s_c32, t1, t4);
        s_t[0] = (double)t1 - pad;
        s_t[1] = (double)t4 + pad;
      }
    } else if (lane == 0 && warp < 2) {
      s_t[warp] = warp == 0 ? contact_point(km, 1, s_c64) - pad : contact_point(km, 4, s_c64) + pad;
    }
  }
  __syncthreads();
  if (tid >= TS_ORB) return;
  R* o = orb + (size_t)pv * TS_ORB;
  if (tid == 0) {
    kstat[pv] = km;
    kstat[npv + pv] = kx;
  }
  if (!valid) {
    o[tid] = R(0);
    return;
  }
  const double t1 = s_t[0], t4 = s_t[1];
  R v = R(0);
  if (tid < 10) {
    v = SPLIT ? (R)s_c32[tid] : (R)s_c64[tid];
  } else {
    const float p_hi = __double2float_rn(pp);
    const double d0 = t0[pv] - t_ref;
    const float d0h = __double2float_rn(d0);
    const double err = ldexp(1.0, -21) * (t_absmax + fabs(d0) + pp) + 1e-9;
    switch (tid) {
      case 10: v = (R)t1; break;
      case 11: v = (R)t4; break;
      case 12: v = (R)km; break;
      case 13: v = (R)(1.0 / (1.0 + km)); break;
      case 14: v = (R)(1.0 - kx); break;
      case 15: v = R(1); break;
      case 16: v = (R)p_hi; break;
      case 17: v = (R)__double2float_rn(pp - (double)p_hi); break;
      case 18: v = (R)__double2float_rn(1.0 / pp); break;
      case 19: v = (R)d0h; break;
      case 20: v = (R)__double2float_rn(d0 - (double)d0h); break;
      case 21: v = (R)err; break;
      case 22: v = (t4 + 2 * err >= 0.5 * pp || t1 - 2 * err <= -0.5 * pp) ? R(1) : R(0); break;
      default: v = R(0);
    }
  }
  o[tid] = v;
}

constexpr int TS_L2_ROWS = 16;   // g rows of the 2D table per LD block

// ---------------------------------------------------------------------------
// Fused TS prologue for the default 2D table (no weight table): one launch
// does the work of ld_tables_kernel, ts_prepare_kernel and ts_ldm2d_kernel.
//   blocks [0, npv): per-pv blocks: mean and largest k, orbit, box, record;
//   blocks [npv, ...): LD blocks (pv, chunk of TS_L2_ROWS rows, chunk of
//     channels): the same k statistics (the same reduction, so the same
//     bits), the channels' LD profiles (from the law's coefficients, or read
//     from ldp for a host-evaluated law) staged in shared memory, the 2D
//     table rows at kmean, the LD means by 16-byte shared-memory loads; the
//     blocks of the first row chunk also write the channel records (afac,
//     k - kmean, 1/istar) with istar from the law's integral or the
//     reference's 200-point trapezoid (rrmodel.py:222-227).
// The orbit blocks come first in the grid, so their serial chains start at
// once and the LD blocks fill the SMs around them.
// ---------------------------------------------------------------------------
constexpr int TSP_MAXPAR = 16;

template <typename R>
struct TsProArgs {
  const double *k, *t0, *p, *a, *inc, *e, *w;
  const double *ldc, *mu, *ze;   // law >= 0: coefficients [npv, npb, npar] and the mu grid
  const R *ldp, *istar;          // law < 0: host-evaluated profiles and integrals
  int law, npar, npv, npb, nz, ng, nrc, ncc;
  double exptime0, t_ref, t_absmax;
  R *orb, *ch, *ldm;
};

// Mean and largest radius ratio of pv by warps 0-2 of the block (strided
// sums, shuffle trees, then the three warp results in order): every block
// that calls it gets the same bits.
__device__ __forceinline__ void ts_kstats(const double* __restrict__ kp, int npb, double* s_sum, double* s_max) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (warp < 3) {
    double sm = 0.0, mx = -INFINITY;
    for (int b = tid; b < npb; b += 96) {
      const double kb = kp[b];
      sm += kb;
      mx = fmax(mx, kb);
    }
    for (int o = 16; o > 0; o >>= 1) {
      sm += __shfl_xor_sync(0xffffffffu, sm, o);
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    if (lane == 0) {
      s_sum[warp] = sm;
      s_max[warp] = mx;
    }
  }
}

template <typename R, bool SPLIT>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 8 : 4) ts_prologue_kernel(TsProArgs<R> P) {
  __shared__ double s_sum[3], s_max[3];
  __shared__ __align__(16) R Wr[TS_L2_ROWS][64];
  __shared__ R s_mu[64];
  __shared__ R s_cf[128][TSP_MAXPAR + 1];   // each thread's channel coefficients (law >= 0)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int npb = P.npb, nz = P.nz, ng = P.ng;
  if ((int)blockIdx.x < P.npv) {
    // ---- per-pv block: k statistics, orbit, box, record ----
    __shared__ double s_c64[10];
    __shared__ float s_c32[10];
    __shared__ double s_t[2];
    const int pv = blockIdx.x;
    const double av = P.a[pv], ev = P.e[pv], pp = P.p[pv];
    const bool valid = !(isnan(av) || av <= 1.0 || ev < 0.0);
    if (warp == 3) {
      if (lane == 0 && valid) {
        if (SPLIT)
          solve2d_conj_f32(pp, av, P.inc[pv], ev, P.w[pv], s_c32);
        else
          solve2d_conj(pp, av, P.inc[pv], ev, P.w[pv], s_c64);
      }
    } else {
      ts_kstats(P.k + (size_t)pv * npb, npb, s_sum, s_max);
    }
    __syncthreads();
    const double km = ((s_sum[0] + s_sum[1]) + s_sum[2]) / npb;
    const double kx = fmax(fmax(s_max[0], s_max[1]), s_max[2]);
    const double pad = 0.0015 + P.exptime0;
    if (valid) {
      if (SPLIT) {
        if (tid == 0) {
          float t1, t4;
          contact_points14_f32((float)km, s_c32, t1, t4);
          s_t[0] = (double)t1 - pad;
          s_t[1] = (double)t4 + pad;
        }
      } else if (lane == 0 && warp < 2) {
        s_t[warp] = warp == 0 ? contact_point(km, 1, s_c64) - pad : contact_point(km, 4, s_c64) + pad;
      }
    }
    __syncthreads();
    if (tid >= TS_ORB) return;
    R* o = P.orb + (size_t)pv * TS_ORB;
    if (!valid) {
      o[tid] = R(0);
      return;
    }
    const double t1 = s_t[0], t4 = s_t[1];
    R v = R(0);
    if (tid < 10) {
      v = SPLIT ? (R)s_c32[tid] : (R)s_c64[tid];
    } else {
      const float p_hi = __double2float_rn(pp);
      const double d0 = P.t0[pv] - P.t_ref;
      const float d0h = __double2float_rn(d0);
      const double err = ldexp(1.0, -21) * (P.t_absmax + fabs(d0) + pp) + 1e-9;
      switch (tid) {
        case 10: v = (R)t1; break;
        case 11: v = (R)t4; break;
        case 12: v = (R)km; break;
        case 13: v = (R)(1.0 / (1.0 + km)); break;
        case 14: v = (R)(1.0 - kx); break;
        case 15: v = R(1); break;
        case 16: v = (R)p_hi; break;
        case 17: v = (R)__double2float_rn(pp - (double)p_hi); break;
        case 18: v = (R)__double2float_rn(1.0 / pp); break;
        case 19: v = (R)d0h; break;
        case 20: v = (R)__double2float_rn(d0 - (double)d0h); break;
        case 21: v = (R)err; break;
        case 22: v = (t4 + 2 * err >= 0.5 * pp || t1 - 2 * err <= -0.5 * pp) ? R(1) : R(0); break;
        default: v = R(0);
      }
    }
    o[tid] = v;
    return;
  }
  // ---- LD block (pv, row chunk rc, channel chunk cc) ----
  const int j = (int)blockIdx.x - P.npv;
  const int per_pv = P.nrc * P.ncc;
  const int pv = j / per_pv, rc = (j % per_pv) / P.ncc, cc = j % P.ncc;
  const int g0 = rc * TS_L2_ROWS, nr = min(TS_L2_ROWS, ng - g0);
  const int cpb = (npb + P.ncc - 1) / P.ncc;          // channels of this block
  const int cb0 = cc * cpb, cb1 = min(npb, cb0 + cpb);
  const int nz4 = (nz + 3) & ~3;                       // z padded to whole 4-vectors (zero weights)
  const double* kp = P.k + (size_t)pv * npb;
  if (P.law >= 0)   // a host-evaluated law (law < 0) passes no mu grid
    for (int i = tid; i < nz4; i += blockDim.x) s_mu[i] = i < nz ? (R)P.mu[i] : R(0);
  ts_kstats(kp, npb, s_sum, s_max);
  __syncthreads();
  const double k = ((s_sum[0] + s_sum[1]) + s_sum[2]) / npb;
  // the 2D table rows at kmean (calculate_weights_2d, common.py:153-185): a
  // warp per row, lanes over z (z and z + 32), the differences through
  // shuffles, the row sum by a shuffle tree
  const double gstep = (1.0 - 1e-7) / (double)(ng - 1);
  const float kf = (float)k, gstep_f = (float)gstep, opk_f = (float)(1.0 + k);
  for (int r = warp; r < nr; r += blockDim.x >> 5) {
    const int g = g0 + r;
    const bool f64 = !SPLIT || g == ng - 1;   // the split path's grazing last row: FP64 areas
    if (SPLIT && !f64) {
      // FP32 kite areas and differences, the row sum by a shuffle tree
      float af[2];
#pragma unroll
      for (int h = 0; h < 2; ++h)
        af[h] = cci_kite_f32((float)P.ze[min(lane + 32 * h, nz - 1)], kf, (float)g * gstep_f * opk_f);
      const float q0 = __shfl_up_sync(0xffffffffu, af[0], 1), q1 = __shfl_up_sync(0xffffffffu, af[1], 1);
      const float l0 = __shfl_sync(0xffffffffu, af[0], 31);
      const float df0 = lane == 0 ? af[0] : af[0] - q0;
      const float df1 = nz <= 32 ? 0.0f : (lane == 0 ? af[1] - l0 : af[1] - q1);
      float sf = df0 + df1;
      for (int o = 16; o > 0; o >>= 1) sf += __shfl_xor_sync(0xffffffffu, sf, o);
      if (sf > 0.0f) {
        const float is = 1.0f / sf;
        if (lane < nz) Wr[r][lane] = (R)(df0 * is);
        if (lane + 32 < nz) Wr[r][lane + 32] = (R)(df1 * is);
        for (int z = nz + lane; z < nz4; z += 32) Wr[r][z] = R(0);
        continue;
      }
      // a row left without area in FP32: the FP64 path below
    }
    const double gg = (g == ng - 1) ? 1.0 - 1e-7 : (double)g * gstep;
    double av[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int z = lane + 32 * h;
      const int zc = min(z, nz - 1);          // lanes past the grid repeat the last area: zero difference
      av[h] = f64 ? cci_acos(P.ze[zc], k, gg * (1.0 + k))
                  : (double)cci_kite_f32((float)P.ze[zc], kf, (float)g * gstep_f * opk_f);
    }
    const double prev0 = __shfl_up_sync(0xffffffffu, av[0], 1);
    const double prev1 = __shfl_up_sync(0xffffffffu, av[1], 1);
    const double last0 = __shfl_sync(0xffffffffu, av[0], 31);
    double d[2];
    d[0] = lane == 0 ? av[0] : av[0] - prev0;
    d[1] = lane == 0 ? av[1] - last0 : av[1] - prev1;
    if (nz <= 32) d[1] = 0.0;
    if (f64) {
      if constexpr (!SPLIT) {
        // the plain path sums the differences in order, as the reference does
        double sm = 0.0;
        for (int z = 0; z < nz; ++z) sm += __shfl_sync(0xffffffffu, d[z >> 5], z & 31);
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (lane + 32 * h < nz) Wr[r][lane + 32 * h] = (R)(d[h] / sm);
      } else {
        double sd = d[0] + d[1];
        for (int o = 16; o > 0; o >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, o);
        const double is = 1.0 / sd;
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (lane + 32 * h < nz) Wr[r][lane + 32 * h] = (R)(d[h] * is);
      }
    } else {
      const float df0 = (float)d[0], df1 = (float)d[1];
      float sf = df0 + df1;
      for (int o = 16; o > 0; o >>= 1) sf += __shfl_xor_sync(0xffffffffu, sf, o);
      if (!(sf > 0.0f)) {
        // a row left without area in FP32: FP64 areas
        double a2[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) a2[h] = cci_acos(P.ze[min(lane + 32 * h, nz - 1)], k, gg * (1.0 + k));
        const double q0 = __shfl_up_sync(0xffffffffu, a2[0], 1), q1 = __shfl_up_sync(0xffffffffu, a2[1], 1);
        const double l0 = __shfl_sync(0xffffffffu, a2[0], 31);
        double e[2];
        e[0] = lane == 0 ? a2[0] : a2[0] - q0;
        e[1] = nz <= 32 ? 0.0 : (lane == 0 ? a2[1] - l0 : a2[1] - q1);
        double sd = e[0] + e[1];
        for (int o = 16; o > 0; o >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, o);
        const double is = 1.0 / sd;
#pragma unroll
        for (int h = 0; h < 2; ++h)
          if (lane + 32 * h < nz) Wr[r][lane + 32 * h] = (R)(e[h] * is);
      } else {
        const float is = 1.0f / sf;
        if (lane < nz) Wr[r][lane] = (R)(df0 * is);
        if (lane + 32 < nz) Wr[r][lane + 32] = (R)(df1 * is);
      }
    }
    for (int z = nz + lane; z < nz4; z += 32) Wr[r][z] = R(0);
  }
  __syncthreads();
  // thread t <-> channel cb0 + t (+ 128 ...): the channel record (first row
  // chunk) and the LD means, the profile evaluated on the fly (or read for a
  // host-evaluated law), four z at a time against the rows' weights
  const bool analytic = P.law == LD_UNIFORM || P.law == LD_LINEAR || P.law == LD_QUADRATIC ||
                        P.law == LD_QUADRATIC_TRI || P.law == LD_POWER_2;   // ld_integral's laws
  if (rc == 0 && P.law >= 0 && !analytic) {
    // 2*pi*trapezoid(z*I(mu(z)), z), mu = linspace(1, 0, 200): a warp per channel
    for (int b = cb0 + warp; b < cb1; b += blockDim.x >> 5) {
      R* cf = s_cf[warp];   // the warp's channel (the rows are reused per thread below, after a barrier)
      const double* src = P.ldc + ((size_t)pv * npb + b) * P.npar;
      if (lane < P.npar) cf[lane] = (R)src[lane];
      __syncwarp();
      constexpr int NT = 200;
      R sm = R(0);
      for (int i = lane + 1; i < NT; i += 32) {
        const R m0 = R(NT - i) / R(NT - 1), m1 = R(NT - 1 - i) / R(NT - 1);
        const R z0 = sqrt(R(1) - m0 * m0), z1 = sqrt(R(1) - m1 * m1);
        sm += (z1 - z0) * (z1 * ld_value<R>(P.law, m1, cf, P.npar) + z0 * ld_value<R>(P.law, m0, cf, P.npar)) /
              R(2);
      }
      for (int o = 16; o > 0; o >>= 1) sm += __shfl_xor_sync(0xffffffffu, sm, o);
      if (lane == 0) P.ch[((size_t)pv * npb + b) * TS_CH + 2] = R(2.0 * PI) * sm;   // istar, inverted below
      __syncwarp();
    }
    __syncthreads();
  }
  for (int b = cb0 + tid; b < cb1; b += blockDim.x) {
    R* cf = s_cf[tid];
    if (P.law >= 0) {
      const double* src = P.ldc + ((size_t)pv * npb + b) * P.npar;
      for (int q = 0; q < P.npar; ++q) cf[q] = (R)src[q];
    }
    if (rc == 0) {
      R is;
      if (P.law < 0)
        is = P.istar[(size_t)pv * npb + b];
      else if (analytic)
        ld_integral<R>(P.law, cf, is);
      else
        is = P.ch[((size_t)pv * npb + b) * TS_CH + 2];
      R* cr = P.ch + ((size_t)pv * npb + b) * TS_CH;
      const double kb = kp[b];
      cr[0] = (R)(kb * kb / (k * k));
      cr[1] = (R)(kb - k);
      cr[2] = isfinite((double)is) ? R(1) / is : R(CUDART_NAN);
      cr[3] = R(0);
    }
    R acc[TS_L2_ROWS];
#pragma unroll
    for (int r = 0; r < TS_L2_ROWS; ++r) acc[r] = R(0);
    const R* lp = P.law < 0 ? P.ldp + ((size_t)pv * npb + b) * nz : nullptr;
    for (int z = 0; z < nz4; z += 4) {
      R x[4];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        x[q] = z + q >= nz ? R(0) : (P.law >= 0 ? ld_value<R>(P.law, s_mu[z + q], cf, P.npar) : __ldg(lp + z + q));
#pragma unroll
      for (int r = 0; r < TS_L2_ROWS; ++r) {
        R a = acc[r];
        if constexpr (sizeof(R) == 4) {
          const float4 wv = *reinterpret_cast<const float4*>(&Wr[r][z]);
          a += wv.x * x[0];
          a += wv.y * x[1];
          a += wv.z * x[2];
          a += wv.w * x[3];
        } else {
          const double2 w0 = *reinterpret_cast<const double2*>(&Wr[r][z]);
          const double2 w1 = *reinterpret_cast<const double2*>(&Wr[r][z + 2]);
          a += w0.x * x[0];
          a += w0.y * x[1];
          a += w1.x * x[2];
          a += w1.y * x[3];
        }
        acc[r] = a;
      }
    }
    R* out = P.ldm + ((size_t)pv * npb + b) * ng + g0;
#pragma unroll
    for (int r = 0; r < TS_L2_ROWS; ++r)
      if (r < nr) out[r] = acc[r];
  }
}

// Flux launch: blocks of TSF_WARPS warps, each a range of at most 32
// consecutive tiles of one pv (grid x: tile ranges, y/z: pv), done by
// ts_range.  The pv's record is staged in shared memory.
constexpr int TSF_WARPS = 4;
template <typename R, bool SPLIT>
__global__ void __launch_bounds__(TSF_WARPS * 32) ts_flux_kernel(TsArgs<R> A, int npv, int chunk) {
  __shared__ __align__(16) TsSmem<R> S;
  __shared__ R s_o[TS_ORB];
  const int pv = blockIdx.y + 65535 * blockIdx.z;
  if (pv >= npv) return;   // block-uniform
  const int ntiles = (A.npt + TS_TILE - 1) / TS_TILE;
  const int tb0 = blockIdx.x * chunk, tb1 = min(ntiles, tb0 + chunk);
  if (threadIdx.x < TS_ORB) s_o[threadIdx.x] = A.orb[(size_t)pv * TS_ORB + threadIdx.x];
  __syncthreads();
  ts_range<R, SPLIT>(A, pv, tb0, tb1, s_o, S);
}

struct TsTables {
  void *orb, *ch, *ldm;
  double* kstat;
};

static TsTables carve_ts(void* ws, bool split, int npv, int npb, int ng) {
  const size_t r = split ? sizeof(float) : sizeof(double);
  Carve cv(ws);
  TsTables t;
  t.orb = cv.take<char>(r * (size_t)npv * TS_ORB);
  t.ch = cv.take<char>(r * (size_t)npv * npb * TS_CH);
  t.ldm = cv.take<char>(r * (size_t)npv * npb * ng);
  t.kstat = cv.take<double>((size_t)npv * 2);
  return t;
}

}  // namespace rr

using namespace rr;

extern "C" {

size_t rr_ts_workspace_bytes(int split, int npv, int npb, int ng) {
  Carve c(nullptr);
  const size_t r = split ? sizeof(float) : sizeof(double);
  c.take<char>(r * (size_t)npv * TS_ORB);
  c.take<char>(r * (size_t)npv * npb * TS_CH);
  c.take<char>(r * (size_t)npv * npb * ng);
  c.take<double>((size_t)npv * 2);
  return c.used + 256;
}

void rr_ts_tables(void* workspace, int split, int npv, int npb, int ng, const void** orb, const void** ch,
                  const void** ldm) {
  TsTables t = carve_ts(workspace, split != 0, npv, npb, ng);
  if (orb) *orb = t.orb;
  if (ch) *ch = t.ch;
  if (ldm) *ldm = t.ldm;
}

}  // extern "C"

template <typename R, bool SPLIT>
static int ts_prepare_impl(double t_ref, double t_absmax, const double* k, const double* t0, const double* p,
                           const double* a, const double* inc, const double* e, const double* w, int npv, int npb,
                           double exptime0, const R* ldp, const R* istar, const R* weights, int nk, int ng, int nz,
                           double dk, double kmin, double kmax, const double* z_edges, void* workspace,
                           size_t workspace_bytes, cudaStream_t s, int law = -1, const double* ldc = nullptr,
                           int npar = 0, const double* mu = nullptr) {
  (void)workspace_bytes;
  if (law >= LD_NLAWS || (law >= 0 && (!ldc || !mu || npar < 0 || npar > TSP_MAXPAR))) return RR_ERR_ARG;
  if (law < 0 && (!ldp || !istar)) return RR_ERR_ARG;
  TsTables t = carve_ts(workspace, SPLIT, npv, npb, ng);
  R* orb = static_cast<R*>(t.orb);
  R* ch = static_cast<R*>(t.ch);
  R* ldm = static_cast<R*>(t.ldm);
  if (weights == nullptr) {
    // the reference's default: the 2D table at kmean, all in one launch
    TsProArgs<R> P{};
    P.k = k; P.t0 = t0; P.p = p; P.a = a; P.inc = inc; P.e = e; P.w = w;
    P.ldc = ldc; P.mu = mu; P.ze = z_edges; P.ldp = ldp; P.istar = istar;
    P.law = law; P.npar = npar; P.npv = npv; P.npb = npb; P.nz = nz; P.ng = ng;
    P.nrc = (ng + TS_L2_ROWS - 1) / TS_L2_ROWS;
    // the split path spreads the channels over blocks of 128 (its FP32 areas
    // are cheap to repeat); the plain path computes its FP64 areas once per
    // row chunk and loops over all channels in the block
    P.ncc = SPLIT ? (npb + 127) / 128 : 1;
    P.exptime0 = exptime0; P.t_ref = t_ref; P.t_absmax = t_absmax;
    P.orb = orb; P.ch = ch; P.ldm = ldm;
    const long long nblk = (long long)npv + (long long)npv * P.nrc * P.ncc;
    ts_prologue_kernel<R, SPLIT><<<(unsigned)nblk, 128, 0, s>>>(P);
    return check_launch("rr_ts_prepare");
  }
  if (ldp == nullptr || istar == nullptr) return RR_ERR_ARG;
  ts_prepare_kernel<R, SPLIT><<<npv, TS_PREP_THREADS, 0, s>>>(k, t0, p, a, inc, e, w, istar, npv, npb, exptime0,
                                                             t_ref, t_absmax, orb, ch, t.kstat);
  // LD means at kmean: the 3D table with the TS rule (kmin <= kmean <= max k)
  if constexpr (SPLIT) {
    launch_ldm_f32(ldp, npv, npb, nz, t.kstat, 1, weights, nk, ng, dk, kmin, kmax, z_edges, 1, t.kstat + npv, ldm,
                   s);
  } else {
    launch_ldm_f64(ldp, npv, npb, nz, t.kstat, 1, weights, nk, ng, dk, kmin, kmax, z_edges, 1, t.kstat + npv, ldm,
                   s);
  }
  return check_launch("rr_ts_prepare");
}

template <typename R, bool SPLIT>
static int ts_flux_impl(const double* times, const float* times_ff, int npt, const double* t0, const double* p,
                        int npv, int npb, int nsamples0, double exptime0, int ng, double dg, void* workspace, R* flux,
                        int ldflux, cudaStream_t s, int pv0 = 0, int pv1 = -1, const double* tiles64 = nullptr) {
  TsTables t = carve_ts(workspace, SPLIT, npv, npb, ng);
  if (pv1 < 0) pv1 = npv;
  TsArgs<R> A{};
  A.times = times;
  A.times_ff = reinterpret_cast<const float2*>(times_ff);
  A.t0 = t0 ? t0 + pv0 : nullptr;
  A.p = p ? p + pv0 : nullptr;
  // the range's records: the kernel indexes pv from 0 within the range
  A.orb = static_cast<const R*>(t.orb) + (size_t)pv0 * TS_ORB;
  A.ch = static_cast<const R*>(t.ch) + (size_t)pv0 * npb * TS_CH;
  A.ldm = static_cast<const R*>(t.ldm) + (size_t)pv0 * npb * ng;
  npv = pv1 - pv0;
  A.flux = flux;
  A.ldflux = ldflux;
  A.npt = npt; A.npb = npb; A.ng = ng; A.nsamples0 = nsamples0;
  A.exptime0 = exptime0; A.dg = dg; A.tiles64 = tiles64;
  // tile ranges of up to 32 tiles, shorter when the launch would have fewer
  // than about 64 blocks of 4 warps per SM: the short blocks spread the
  // tiles that hold a transit over the SMs (measured: single-tile blocks beat
  // 16-tile ones by 10 % on 64 pv x 200 channels x 19,700 times)
  const long long ntiles = (npt + TS_TILE - 1) / TS_TILE;
  const long long target = (long long)sm_count() * 64;
  long long chunk = ntiles * npv / target;
  chunk = chunk < 1 ? 1 : (chunk > 32 ? 32 : chunk);
  const long long bx = (ntiles + chunk - 1) / chunk;
  dim3 fg((unsigned)bx, npv < 65535 ? npv : 65535, (npv + 65534) / 65535);
  ts_flux_kernel<R, SPLIT><<<fg, TSF_WARPS * 32, 0, s>>>(A, npv, (int)chunk);
  return check_launch("rr_ts_flux");
}

static int ts_check(int npt, int npv, int npb, int ng, int nz, int nsamples0, int ldflux, int nk, const void* weights) {
  if (npt < 0 || npv < 0 || npb < 1 || ng < 2 || ng > 4096 || nz < 1 || nz > 64 || nsamples0 < 1 || ldflux < npt ||
      (weights && nk < 2))
    return RR_ERR_ARG;
  return RR_OK;
}

extern "C" {

int rr_ts_f64(const double* times, int npt, const double* k, const double* t0, const double* p, const double* a,
              const double* inc, const double* e, const double* w, int npv, int npb, int nsamples0,
              double exptime0, const double* ldp, const double* istar, const double* weights, int nk, int ng,
              int nz, double dk, double kmin, double kmax, double dg, const double* z_edges, void* workspace,
              size_t workspace_bytes, double* flux, int ldflux, void* stream) {
  int st = ts_check(npt, npv, npb, ng, nz, nsamples0, ldflux, nk, weights);
  if (st) return st;
  if (npv == 0 || npt == 0) return RR_OK;
  if (workspace_bytes < rr_ts_workspace_bytes(0, npv, npb, ng)) return RR_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  st = ts_prepare_impl<double, false>(0.0, 0.0, k, t0, p, a, inc, e, w, npv, npb, exptime0, ldp, istar, weights, nk,
                                      ng, nz, dk, kmin, kmax, z_edges, workspace, workspace_bytes, s);
  if (st) return st;
  return ts_flux_impl<double, false>(times, nullptr, npt, t0, p, npv, npb, nsamples0, exptime0, ng, dg, workspace,
                                     flux, ldflux, s);
}

int rr_ts_prepare_split_ld(int law, const double* ldc, int npar, const double* mu, double t_ref, double t_absmax,
                           const double* k, const double* t0, const double* p, const double* a, const double* inc,
                           const double* e, const double* w, int npv, int npb, double exptime0, int ng, int nz,
                           const double* z_edges, void* workspace, size_t workspace_bytes, void* stream) {
  int st = ts_check(0, npv, npb, ng, nz, 1, 0, 0, nullptr);
  if (st) return st;
  if (law < 0 || law >= LD_NLAWS) return RR_ERR_LAW;
  if (npv == 0) return RR_OK;
  if (workspace_bytes < rr_ts_workspace_bytes(1, npv, npb, ng)) return RR_ERR_WORKSPACE;
  return ts_prepare_impl<float, true>(t_ref, t_absmax, k, t0, p, a, inc, e, w, npv, npb, exptime0, nullptr, nullptr,
                                      nullptr, 0, ng, nz, 0.0, 0.0, 0.0, z_edges, workspace, workspace_bytes,
                                      as_stream(stream), law, ldc, npar, mu);
}

int rr_ts_prepare_f64_ld(int law, const double* ldc, int npar, const double* mu, const double* k, const double* t0,
                         const double* p, const double* a, const double* inc, const double* e, const double* w,
                         int npv, int npb, double exptime0, int ng, int nz, const double* z_edges, void* workspace,
                         size_t workspace_bytes, void* stream) {
  int st = ts_check(0, npv, npb, ng, nz, 1, 0, 0, nullptr);
  if (st) return st;
  if (law < 0 || law >= LD_NLAWS) return RR_ERR_LAW;
  if (npv == 0) return RR_OK;
  if (workspace_bytes < rr_ts_workspace_bytes(0, npv, npb, ng)) return RR_ERR_WORKSPACE;
  return ts_prepare_impl<double, false>(0.0, 0.0, k, t0, p, a, inc, e, w, npv, npb, exptime0, nullptr, nullptr,
                                        nullptr, 0, ng, nz, 0.0, 0.0, 0.0, z_edges, workspace, workspace_bytes,
                                        as_stream(stream), law, ldc, npar, mu);
}

int rr_ts_flux_f64(const double* times, int npt, const double* t0, const double* p, int npv, int npb, int nsamples0,
                   double exptime0, int ng, double dg, const void* workspace, double* flux, int ldflux,
                   void* stream) {
  int st = ts_check(npt, npv, npb, ng, 1, nsamples0, ldflux, 0, nullptr);
  if (st) return st;
  if (npv == 0 || npt == 0) return RR_OK;
  return ts_flux_impl<double, false>(times, nullptr, npt, t0, p, npv, npb, nsamples0, exptime0, ng, dg,
                                     const_cast<void*>(workspace), flux, ldflux, as_stream(stream));
}

int rr_ts_flux_f64_culled(const double* times, const double* tiles64, int npt, const double* t0, const double* p,
                          int npv, int npb, int nsamples0, double exptime0, int ng, double dg, const void* workspace,
                          double* flux, int ldflux, void* stream) {
  int st = ts_check(npt, npv, npb, ng, 1, nsamples0, ldflux, 0, nullptr);
  if (st) return st;
  if (npv == 0 || npt == 0) return RR_OK;
  if (!tiles64) return RR_ERR_ARG;
  return ts_flux_impl<double, false>(times, nullptr, npt, t0, p, npv, npb, nsamples0, exptime0, ng, dg,
                                     const_cast<void*>(workspace), flux, ldflux, as_stream(stream), 0, -1, tiles64);
}

int rr_ts_prepare_split(double t_ref, double t_absmax, const double* k, const double* t0, const double* p,
                        const double* a, const double* inc, const double* e, const double* w, int npv, int npb,
                        double exptime0, const float* ldp, const float* istar, const float* weights, int nk, int ng,
                        int nz, double dk, double kmin, double kmax, const double* z_edges, void* workspace,
                        size_t workspace_bytes, void* stream) {
  int st = ts_check(0, npv, npb, ng, nz, 1, 0, nk, weights);
  if (st) return st;
  if (npv == 0) return RR_OK;
  if (workspace_bytes < rr_ts_workspace_bytes(1, npv, npb, ng)) return RR_ERR_WORKSPACE;
  return ts_prepare_impl<float, true>(t_ref, t_absmax, k, t0, p, a, inc, e, w, npv, npb, exptime0, ldp, istar,
                                      weights, nk, ng, nz, dk, kmin, kmax, z_edges, workspace, workspace_bytes,
                                      as_stream(stream));
}

int rr_ts_flux_split(const float* times_ff, int npt, int npv, int npb, int nsamples0, double exptime0, int ng,
                     double dg, const void* workspace, float* flux, int ldflux, void* stream) {
  int st = ts_check(npt, npv, npb, ng, 1, nsamples0, ldflux, 0, nullptr);
  if (st) return st;
  if (npv == 0 || npt == 0) return RR_OK;
  return ts_flux_impl<float, true>(nullptr, times_ff, npt, nullptr, nullptr, npv, npb, nsamples0, exptime0, ng, dg,
                                   const_cast<void*>(workspace), flux, ldflux, as_stream(stream));
}

int rr_ts_flux_split_range(const float* times_ff, int npt, int npv, int npb, int nsamples0, double exptime0, int ng,
                           double dg, const void* workspace, int pv0, int pv1, float* flux, int ldflux, void* stream) {
  int st = ts_check(npt, npv, npb, ng, 1, nsamples0, ldflux, 0, nullptr);
  if (st) return st;
  if (pv0 < 0 || pv1 > npv || pv0 > pv1) return RR_ERR_ARG;
  if (pv0 == pv1 || npt == 0) return RR_OK;
  return ts_flux_impl<float, true>(nullptr, times_ff, npt, nullptr, nullptr, npv, npb, nsamples0, exptime0, ng, dg,
                                   const_cast<void*>(workspace), flux, ldflux, as_stream(stream), pv0, pv1);
}

int rr_ts_split(const float* times_ff, double t_ref, double t_absmax, int npt, const double* k, const double* t0,
                const double* p, const double* a, const double* inc, const double* e, const double* w, int npv,
                int npb, int nsamples0, double exptime0, const float* ldp, const float* istar,
                const float* weights, int nk, int ng, int nz, double dk, double kmin, double kmax, double dg,
                const double* z_edges, void* workspace, size_t workspace_bytes, float* flux, int ldflux,
                void* stream) {
  int st = ts_check(npt, npv, npb, ng, nz, nsamples0, ldflux, nk, weights);
  if (st) return st;
  if (npv == 0 || npt == 0) return RR_OK;
  st = rr_ts_prepare_split(t_ref, t_absmax, k, t0, p, a, inc, e, w, npv, npb, exptime0, ldp, istar, weights, nk, ng,
                           nz, dk, kmin, kmax, z_edges, workspace, workspace_bytes, stream);
  if (st) return st;
  return rr_ts_flux_split(times_ff, npt, npv, npb, nsamples0, exptime0, ng, dg, workspace, flux, ldflux, stream);
}

}  // extern "C"
