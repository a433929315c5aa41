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
#include <cmath>

#include "rr_device.cuh"
#include "rr_internal.h"

namespace rr {

constexpr int TS_ORB = 32;    // per-pv record (R)
// record fields: c[0..9], [10] t1, [11] t4, [12] kmean, [13] 1/(1+kmean),
// [14] 1 - max(k), [15] valid, [16] p_hi, [17] p_lo, [18] 1/p, [19] d0_hi,
// [20] d0_lo, [21] fast-test error bound, [22] wide flag
constexpr int TS_CH = 4;      // per-channel record: afac, k - kmean, 1/istar, unused
constexpr int TS_WARPS = 8;

// Per-pv prologue, one block per pv: kmean (summed in channel order) and max k
// (a block reduction over the channels), the
// channel records, and (thread 0) the orbit and bounding box.  The split path
// finds the contact points in FP32: they only place the padded box.
constexpr int TS_PREP_THREADS = 128;
template <typename R>
__global__ void __launch_bounds__(TS_PREP_THREADS)
ts_prepare_kernel(const double* __restrict__ k, const double* __restrict__ t0, const double* __restrict__ p,
                  const double* __restrict__ a, const double* __restrict__ inc, const double* __restrict__ e,
                  const double* __restrict__ w, const R* __restrict__ istar, int npv, int npb, double exptime0,
                  double t_ref, double t_absmax, R* __restrict__ orb, R* __restrict__ ch,
                  double* __restrict__ kstat) {
  __shared__ double s_kx[TS_PREP_THREADS];
  __shared__ double s_km;
  const int pv = blockIdx.x;
  const double* kp = k + (size_t)pv * npb;
  double kx = -INFINITY;
  for (int b = threadIdx.x; b < npb; b += blockDim.x) kx = fmax(kx, kp[b]);
  s_kx[threadIdx.x] = kx;
  __syncthreads();
  if (threadIdx.x == 0) {
    double km = 0.0;
    for (int b = 0; b < npb; ++b) km += kp[b];
    s_km = km / npb;
    for (int t = 1; t < blockDim.x; ++t) kx = fmax(kx, s_kx[t]);
    s_kx[0] = kx;
  }
  __syncthreads();
  const double km = s_km;
  kx = s_kx[0];
  for (int b = threadIdx.x; b < npb; b += blockDim.x) {
    R* c = ch + ((size_t)pv * npb + b) * TS_CH;
    c[0] = (R)(kp[b] * kp[b] / (km * km));
    c[1] = (R)(kp[b] - km);
    const R is = istar[(size_t)pv * npb + b];
    c[2] = isfinite((double)is) ? R(1) / is : R(CUDART_NAN);
    c[3] = R(0);
  }
  if (threadIdx.x != 0) return;
  kstat[pv] = km;
  kstat[npv + pv] = kx;
  const bool valid = !(isnan(a[pv]) || a[pv] <= 1.0 || e[pv] < 0.0);
  R* o = orb + (size_t)pv * TS_ORB;
  for (int i = 0; i < TS_ORB; ++i) o[i] = R(0);
  o[15] = valid ? R(1) : R(0);
  if (!valid) return;
  double c[10];
  solve2d_conj(p[pv], a[pv], inc[pv], e[pv], w[pv], c);
  const double pad = 0.0015 + exptime0;
  double t1, t4;
  if (sizeof(R) == 4) {
    float cf[10];
    for (int i = 0; i < 10; ++i) cf[i] = (float)c[i];
    t1 = contact_point_f32((float)km, 1, cf) - pad;
    t4 = contact_point_f32((float)km, 4, cf) + pad;
  } else {
    t1 = contact_point(km, 1, c) - pad;
    t4 = contact_point(km, 4, c) + pad;
  }
  for (int i = 0; i < 10; ++i) o[i] = (R)c[i];
  o[10] = (R)t1;
  o[11] = (R)t4;
  o[12] = (R)km;
  o[13] = (R)(1.0 / (1.0 + km));
  o[14] = (R)(1.0 - kx);
  const float p_hi = __double2float_rn(p[pv]);
  o[16] = (R)p_hi;
  o[17] = (R)__double2float_rn(p[pv] - (double)p_hi);
  o[18] = (R)__double2float_rn(1.0 / p[pv]);
  const double d0 = t0[pv] - t_ref;
  const float d0h = __double2float_rn(d0);
  o[19] = (R)d0h;
  o[20] = (R)__double2float_rn(d0 - (double)d0h);
  const double err = ldexp(1.0, -21) * (t_absmax + fabs(d0) + p[pv]) + 1e-9;
  o[21] = (R)err;
  o[22] = (t4 + 2 * err >= 0.5 * p[pv] || t1 - 2 * err <= -0.5 * p[pv]) ? R(1) : R(0);
}

// LD means of the reference's default TS table (calculate_weights_2d at
// kmean, model_trspec.py:50-53): block (pv, chunk of TS_L2_ROWS g rows)
// builds its rows of the 2D table (areas at every (g, z) in parallel, then
// per row the differences and their sum, normalised in FP64) and reduces
// them right away against every channel's LD profile:
//   ldm[pv, b, g] = sum_z W2[g, z] ldp[pv, b, z].
// The plain path takes the areas from the reference's acos form in FP64; the
// split path from the kite form (Agol et al. 2020) in FP32, which is stable
// and 64x cheaper on GB300 (table error ~1e-7 relative at k = 0.1, ~5e-9 in
// flux; ~2e-7 in flux at k = 0.5).
constexpr int TS_L2_ROWS = 16;
template <typename R>
__global__ void __launch_bounds__(128)
ts_ldm2d_kernel(const R* __restrict__ ldp, int npb, int nz, const double* __restrict__ kmean,
                const double* __restrict__ ze, int ng, R* __restrict__ ldm) {
  __shared__ double A2[TS_L2_ROWS][64];
  __shared__ R Wr[TS_L2_ROWS][65];
  const int pv = blockIdx.x, g0 = blockIdx.y * TS_L2_ROWS;
  const int nr = min(TS_L2_ROWS, ng - g0);
  const double k = kmean[pv];
  const double gstep = (1.0 - 1e-7) / (double)(ng - 1);
  for (int i = threadIdx.x; i < nr * nz; i += blockDim.x) {
    const int r = i / nz, z = i % nz, g = g0 + r;
    const double gg = (g == ng - 1) ? 1.0 - 1e-7 : (double)g * gstep;
    if (sizeof(R) == 4)
      A2[r][z] = (double)cci_kite_f32((float)ze[z], (float)k, (float)(gg * (1.0 + k)));
    else
      A2[r][z] = cci_acos(ze[z], k, gg * (1.0 + k));
  }
  __syncthreads();
  for (int r = threadIdx.x; r < nr; r += blockDim.x) {
    double s = A2[r][0];
    for (int z = 1; z < nz; ++z) s += A2[r][z] - A2[r][z - 1];
    if (sizeof(R) == 4 && (g0 + r == ng - 1 || !(s > 0.0))) {
      // the grazing last row (b = (1 - 1e-7)(1 + k) rounds onto contact in
      // FP32) and any row left without area: FP64 areas
      const int g = g0 + r;
      const double gg = (g == ng - 1) ? 1.0 - 1e-7 : (double)g * gstep;
      for (int z = 0; z < nz; ++z) A2[r][z] = cci_acos(ze[z], k, gg * (1.0 + k));
      s = A2[r][0];
      for (int z = 1; z < nz; ++z) s += A2[r][z] - A2[r][z - 1];
    }
    if (sizeof(R) == 8) {
      Wr[r][0] = (R)(A2[r][0] / s);
      for (int z = 1; z < nz; ++z) Wr[r][z] = (R)((A2[r][z] - A2[r][z - 1]) / s);
    } else {
      const double is = 1.0 / s;
      Wr[r][0] = (R)(A2[r][0] * is);
      for (int z = 1; z < nz; ++z) Wr[r][z] = (R)((A2[r][z] - A2[r][z - 1]) * is);
    }
  }
  __syncthreads();
  const R* lp = ldp + (size_t)pv * npb * nz;
  for (int j = threadIdx.x; j < npb * nr; j += blockDim.x) {
    const int b = j / nr, r = j % nr;
    const R* lb = lp + (size_t)b * nz;
    R d = R(0);
    for (int z = 0; z < nz; ++z) d += Wr[r][z] * __ldg(lb + z);
    ldm[((size_t)pv * npb + b) * ng + g0 + r] = d;
  }
}

// Phase-folded time of point pt (time from the nearest conjunction) of the
// TS kernel: FP32 pairs with error-free transformations in the split path,
// the reference's FP64 fold (model_trspec.py:74-76) in the plain path.
template <typename R, bool SPLIT>
__device__ __forceinline__ R ts_fold(int pt, const double* __restrict__ times, const float2* __restrict__ times_ff,
                                     double tz, double pp, const R* o) {
  if constexpr (SPLIT) {
    const float2 tt = __ldg(times_ff + pt);
    const float d0h = (float)o[19], d0l = (float)o[20], p_hi = (float)o[16], p_lo = (float)o[17];
    float n = floorf(fmaf(tt.x - d0h, (float)o[18], 0.5f));
    float s1, e1, q1, e2, s2, e3;
    two_sum(tt.x, -d0h, s1, e1);
    two_prod(n, p_hi, q1, e2);
    two_sum(s1, -q1, s2, e3);
    float t = s2 + (((e1 + e3) - e2) + (tt.y - d0l) - n * p_lo);
    if (t >= 0.5f * p_hi || t < -0.5f * p_hi) {
      n += (t >= 0.5f * p_hi) ? 1.0f : -1.0f;
      two_prod(n, p_hi, q1, e2);
      two_sum(s1, -q1, s2, e3);
      t = s2 + (((e1 + e3) - e2) + (tt.y - d0l) - n * p_lo);
    }
    return (R)t;
  } else {
    const double t = times[pt];
    const double epoch = floor(__ddiv_rn(__dadd_rn(__dsub_rn(t, tz), __dmul_rn(0.5, pp)), pp));
    return (R)__dsub_rn(t, __dadd_rn(tz, __dmul_rn(epoch, pp)));
  }
}

// One exposure sample at time t from conjunction: z by Horner, the area at
// kmean and its k-derivative, the LD-table row and fraction; false when the
// planet does not occult the star.
template <typename R>
__device__ __forceinline__ bool ts_sample(R t, const R* cc, R kmean, R inv1pk, R inv_dg, int ng, R inner_lim, R& a,
                                          R& dadk, int& gi, R& fr, bool& inner) {
  R x = cc[4], y = cc[9];
  for (int mm = 3; mm >= 0; --mm) {
    x = x * t + cc[mm];
    y = y * t + cc[5 + mm];
  }
  const R z = sqrt(x * x + y * y);
  if (!(z <= R(1) + kmean)) return false;
  R kap;
  a = ccia_star<R>(kmean, z, kap);
  dadk = R(2) * kmean * kap;
  const R gg = z * inv1pk * inv_dg;
  gi = min(max((int)gg, 0), ng - 2);
  fr = gg - (R)gi;
  inner = z <= inner_lim;
  return a != R(0);
}

constexpr int TS_MW = 8;      // LD-table rows a lane keeps weights for
constexpr int TS_SCOLS = 16;  // LD-table columns a warp stages per round

// A block owns a contiguous range of warp tiles (128 points, 4 per lane) of
// one pv.  The range's channel rows are first filled with 1.0, row by row;
// then each warp takes a tile at a time.  In-box points are
// then taken 32 at a time, one per lane, consecutive points in consecutive
// lanes: a lane folds its exposure samples into weights on at most TS_MW
// consecutive rows of the LD-mean tables, since for every channel b
//   sum_s I_b(g_s) area_b(s) = sum_j L_b[j] (afac_b win_j + wout_j + dk_b wd_j)
// (area_b = afac_b a_s fully inside, a_s + dk_b da/dk on the limb), then loops
// over the channels (32 at a time, with their table columns staged in shared
// memory): reads within the channel's table row, coalesced stores.
// Points whose samples span more rows are evaluated afterwards by the whole
// warp, lanes over samples and then over channels.
template <typename R, bool SPLIT>
__global__ void __launch_bounds__(TS_WARPS * 32, sizeof(R) == 4 ? 4 : 2)
ts_flux_kernel(const double* __restrict__ times, const float2* __restrict__ times_ff, int npt,
               const double* __restrict__ t0, const double* __restrict__ p, int npv, int npb, int nsamples0,
               double exptime0, const R* __restrict__ orb_all, const R* __restrict__ ch_all,
               const R* __restrict__ ldm_all, int ng, double dg, R* __restrict__ flux, int ldflux) {
  const unsigned FULL = 0xffffffffu;
  __shared__ R s_tab[TS_WARPS][32 * (TS_SCOLS + 1)];   // per warp: 32 channels x table columns
  __shared__ R s_rec[TS_WARPS][32 * 4];                // per warp: 32 channel records
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pv = blockIdx.y + 65535 * blockIdx.z;
  if (pv >= npv) return;
  const R* o = orb_all + (size_t)pv * TS_ORB;
  const R* ch = ch_all + (size_t)pv * npb * TS_CH;
  const R* ldm = ldm_all + (size_t)pv * npb * ng;     // [npb][ng]
  R* fpv = flux + (size_t)pv * npb * ldflux;
  const bool valid = o[15] != R(0);
  const int ntiles = (npt + 127) / 128;
  const float4* meta = SPLIT ? reinterpret_cast<const float4*>(reinterpret_cast<const float*>(times_ff) +
                                                               time_meta_offset(npt))
                             : nullptr;
  R cc[10];
  for (int i = 0; i < 10; ++i) cc[i] = o[i];
  const R box_lo = o[10], box_hi = o[11], kmean = o[12], inv1pk = o[13], inner_lim = o[14];
  const R inv_dg = R(1) / (R)dg;
  const R ex = (R)exptime0;
  const R inv_ns = R(1) / (R)nsamples0;
  const double tz = SPLIT ? 0.0 : t0[pv], pp = SPLIT ? 0.0 : p[pv];
  const bool vec_ok = ((ldflux & 3) == 0) && ((reinterpret_cast<uintptr_t>(flux) & 15) == 0) && sizeof(R) == 4;

  // The block owns the contiguous tiles [tb0, tb1).  First its warps fill
  // every channel row of that range with ones (NaN for an invalid pv), row by
  // row: each row segment is one contiguous run, so the output stream reaches
  // DRAM in long runs rather than 512-byte pieces scattered over npb rows.
  // After the block barrier, warps take the tiles and overwrite the in-box
  // points.
  const int tpb = (ntiles + gridDim.x - 1) / gridDim.x;
  const int tb0 = blockIdx.x * tpb, tb1 = min(ntiles, tb0 + tpb);
  if (tb0 >= tb1) return;   // block-uniform
  {
    const R fill = valid ? R(1) : R(CUDART_NAN);
    const int p0 = tb0 * 128, p1 = min(npt, tb1 * 128);
    for (int b = warp; b < npb; b += TS_WARPS) {
      R* row = fpv + (size_t)b * ldflux;
      int pt = p0 + lane;
      if constexpr (sizeof(R) == 4) {
        if (vec_ok) {
          const int n4 = (p1 - p0) >> 2;   // whole float4s from p0 (a multiple of 4)
          float4* r4 = reinterpret_cast<float4*>(row + p0);
          for (int i = lane; i < n4; i += 32) __stcs(r4 + i, make_float4(fill, fill, fill, fill));
          pt = p0 + 4 * n4 + lane;
        }
      }
      for (; pt < p1; pt += 32) row[pt] = fill;
    }
  }
  __syncthreads();
  if (!valid) return;       // block-uniform

  for (int tile = tb0 + warp; tile < tb1; tile += TS_WARPS) {
    const int pt0 = tile * 128 + lane * 4;
    // tile cull (split: from the tile summary)
    if (SPLIT && !(o[22] != R(0))) {
      const float4 tm = __ldg(meta + tile);
      const float d0h = (float)o[19], p_hi = (float)o[16], inv_p = (float)o[18], err = (float)o[21];
      const float smin = tm.x - d0h, smax = tm.y - d0h;
      const float flo = (float)box_lo - err, fhi = (float)box_hi + err;
      const float j0 = ceilf((smin - fhi) * inv_p);
      bool hit = false;
      for (int dj = -1; dj <= 1; ++dj) {
        const float jj = j0 + (float)dj;
        hit = hit || (fmaf(jj, p_hi, flo) <= smax && fmaf(jj, p_hi, fhi) >= smin);
      }
      if (!hit) continue;
    }
    // in-box flags of the lane's 4 points
    unsigned inb = 0;
    for (int q = 0; q < 4; ++q) {
      const int pt = pt0 + q;
      if (pt >= npt) continue;
      const R tc = ts_fold<R, SPLIT>(pt, times, times_ff, tz, pp, o);
      if (box_lo <= tc && tc <= box_hi) inb |= 1u << q;
    }
    const unsigned bq0 = __ballot_sync(FULL, inb & 1u), bq1 = __ballot_sync(FULL, inb >> 1 & 1u);
    const unsigned bq2 = __ballot_sync(FULL, inb >> 2 & 1u), bq3 = __ballot_sync(FULL, inb >> 3 & 1u);
    if ((bq0 | bq1 | bq2 | bq3) == 0u) continue;

    for (int r = 0; r < 4; ++r) {
      // lane <-> tile point r*32 + lane, owned in the fill above by lane (r*32+lane)/4
      const int pl = r * 32 + lane;
      const int own = pl >> 2, slot = pl & 3;
      const unsigned bq = slot == 0 ? bq0 : (slot == 1 ? bq1 : (slot == 2 ? bq2 : bq3));
      const bool mine = (bq >> own) & 1u;
      if (!__any_sync(FULL, mine)) continue;
      const int pt = tile * 128 + pl;
      R tc = R(0);
      int jlo = 0, nwin = 0;
      bool act = false, wide = false, any_in = false, any_out = false;
      R win[TS_MW], wout[TS_MW], wd[TS_MW];
      for (int j = 0; j < TS_MW; ++j) win[j] = wout[j] = wd[j] = R(0);
      if (mine) {
        tc = ts_fold<R, SPLIT>(pt, times, times_ff, tz, pp, o);
        // pass 1: the rows the samples touch
        int lo = 0x7fffffff, hi = -1;
        for (int s = 0; s < nsamples0; ++s) {
          const R t = tc + ex * ((R(s) + R(0.5)) * inv_ns - R(0.5));
          R x = cc[4], y = cc[9];
          for (int mm = 3; mm >= 0; --mm) {
            x = x * t + cc[mm];
            y = y * t + cc[5 + mm];
          }
          const R z = sqrt(x * x + y * y);
          if (z <= R(1) + kmean) {
            const int g = min(max((int)(z * inv1pk * inv_dg), 0), ng - 2);
            lo = min(lo, g);
            hi = max(hi, g + 1);
          }
        }
        jlo = lo;
        nwin = hi >= 0 ? hi - lo + 1 : 0;
        wide = nwin > TS_MW;
        // pass 2: the row weights (a row outside the window found in pass 1,
        // possible only through a different rounding of z, sends the point
        // to the warp path below)
        if (hi >= 0 && !wide) {
          for (int s = 0; s < nsamples0; ++s) {
            const R t = tc + ex * ((R(s) + R(0.5)) * inv_ns - R(0.5));
            R a, dadk, fr;
            int gi;
            bool inner;
            if (!ts_sample<R>(t, cc, kmean, inv1pk, inv_dg, ng, inner_lim, a, dadk, gi, fr, inner)) continue;
            const int j0 = gi - jlo;
            if (j0 < 0 || j0 + 1 >= nwin) {
              wide = true;
              act = false;
              break;
            }
            act = true;
#pragma unroll
            for (int j = 0; j < TS_MW; ++j) {
              const R wgt = (j == j0) ? R(1) - fr : ((j == j0 + 1) ? fr : R(0));
              if (inner) {
                win[j] += wgt * a;
              } else {
                wout[j] += wgt * a;
                wd[j] += wgt * dadk;
              }
            }
            any_in |= inner;
            any_out |= !inner;
          }
        }
      }
      const bool w_in = __any_sync(FULL, act && any_in), w_out = __any_sync(FULL, act && any_out);
      if (__any_sync(FULL, act)) {
        const int nrow = act ? nwin : 0;                      // rows jlo .. jlo + nwin - 1 < ng
        const int mrow = __reduce_max_sync(FULL, nrow);       // loop bound, the same in every lane
        // the table columns the warp's lanes read, gmin .. gmax
        const int gmin = __reduce_min_sync(FULL, act ? jlo : 0x7fffffff);
        const int gmax = __reduce_max_sync(FULL, act ? jlo + nwin - 1 : -1);
        const int ncol = gmax - gmin + 1;
        R* stab = s_tab[warp];
        R* srec = s_rec[warp];
        for (int c0 = 0; c0 < npb; c0 += 32) {
          const int nc = min(32, npb - c0);
          // 32 channels at a time: each lane stages one channel's record and,
          // when the warp's columns fit, its table columns; then every lane
          // evaluates its point for the 32 channels from shared memory
          const bool staged = ncol <= TS_SCOLS;
          if (lane < nc) {
            const R* cr = ch + (size_t)(c0 + lane) * TS_CH;
            srec[lane * 4 + 0] = cr[0];
            srec[lane * 4 + 1] = cr[1];
            srec[lane * 4 + 2] = cr[2];
            if (staged) {
              const R* src = ldm + (size_t)(c0 + lane) * ng + gmin;
              for (int j = 0; j < ncol; ++j) stab[lane * (TS_SCOLS + 1) + j] = src[j];
            }
          }
          __syncwarp();
          if (act) {
            for (int c = 0; c < nc; ++c) {
              const R afac = srec[c * 4 + 0], dkb = srec[c * 4 + 1], inv_is = srec[c * 4 + 2];
              const R* Lb = staged ? stab + c * (TS_SCOLS + 1) + (jlo - gmin) : ldm + (size_t)(c0 + c) * ng + jlo;
              R acc_in = R(0), acc_out = R(0), acc_d = R(0);
#pragma unroll
              for (int j = 0; j < TS_MW; ++j) {
                if (j >= mrow) break;
                const R l = (j < nrow) ? Lb[j] : R(0);
                if (w_in) acc_in += l * win[j];
                if (w_out) {
                  acc_out += l * wout[j];
                  acc_d += l * wd[j];
                }
              }
              fpv[(size_t)(c0 + c) * ldflux + pt] =
                  R(1) - (afac * acc_in + acc_out + dkb * acc_d) * inv_is * inv_ns;
            }
          }
          __syncwarp();
        }
      }
      // points whose samples span more than TS_MW rows: the whole warp, one point at a time
      unsigned wm = __ballot_sync(FULL, mine && wide);
      while (wm) {
        const int src = __ffs(wm) - 1;
        wm &= wm - 1;
        const R tcw = __shfl_sync(FULL, tc, src);
        const int ptw = tile * 128 + r * 32 + src;
        for (int s0 = 0; s0 < nsamples0; s0 += 32) {
          const int ns_here = min(32, nsamples0 - s0);
          R a = R(0), dadk = R(0), fr = R(0);
          int gi = 0;
          bool inner = false, ok = false;
          if (lane < ns_here) {
            const R t = tcw + ex * ((R(s0 + lane) + R(0.5)) * inv_ns - R(0.5));
            ok = ts_sample<R>(t, cc, kmean, inv1pk, inv_dg, ng, inner_lim, a, dadk, gi, fr, inner);
          }
          const unsigned okm = __ballot_sync(FULL, ok);
          for (int b0 = 0; b0 < npb; b0 += 32) {
            const int b = b0 + lane;
            const int bb = b < npb ? b : npb - 1;
            const R* cr = ch + (size_t)bb * TS_CH;
            const R afac = cr[0], dkb = cr[1];
            const R* Lb = ldm + (size_t)bb * ng;
            R acc = R(0);
            for (int s = 0; s < ns_here; ++s) {
              if (!(okm >> s & 1u)) continue;
              const int g_s = __shfl_sync(FULL, gi, s);
              const R f_s = __shfl_sync(FULL, fr, s);
              const R a_s = __shfl_sync(FULL, a, s);
              const R d_s = __shfl_sync(FULL, dadk, s);
              const bool in_s = __shfl_sync(FULL, (int)inner, s) != 0;
              const R l0 = Lb[g_s], l1 = Lb[g_s + 1];
              acc += (l0 + f_s * (l1 - l0)) * (in_s ? a_s * afac : a_s + dkb * d_s);
            }
            if (b < npb) {
              R* dst = fpv + (size_t)b * ldflux + ptw;
              // samples beyond the first 32 add to the value already stored
              const R prev = (s0 == 0) ? R(1) : *dst;
              *dst = prev - acc * cr[2] * inv_ns;
            }
          }
          __syncwarp();
        }
      }
    }
  }
}

}  // namespace rr

using namespace rr;

extern "C" {

size_t rr_ts_workspace_bytes(int split, int npv, int npb, int ng) {
  const size_t r = split ? sizeof(float) : sizeof(double);
  Carve c(nullptr);
  c.take<char>(r * (size_t)npv * TS_ORB);
  c.take<char>(r * (size_t)npv * npb * TS_CH);
  c.take<char>(r * (size_t)npv * npb * ng);
  c.take<double>((size_t)npv * 2);
  return c.used + 256;
}

}  // extern "C"

template <typename R, bool SPLIT>
static int ts_impl(const double* times, const float* times_ff, double t_ref, double t_absmax, int npt,
                   const double* k, const double* t0, const double* p, const double* a, const double* inc,
                   const double* e, const double* w, int npv, int npb, int nsamples0, double exptime0,
                   const R* ldp, const R* istar, const R* weights, int nk, int ng, int nz, double dk, double kmin,
                   double kmax, double dg, const double* z_edges, void* workspace, size_t workspace_bytes, R* flux,
                   int ldflux, void* stream) {
  if (npt < 0 || npv < 0 || npb < 1 || ng < 2 || nz < 1 || nz > 64 || nsamples0 < 1 || ldflux < npt ||
      (weights && nk < 2))
    return RR_ERR_ARG;
  if (npv == 0 || npt == 0) return RR_OK;
  if (workspace_bytes < rr_ts_workspace_bytes(SPLIT, npv, npb, ng)) return RR_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  Carve cv(workspace);
  R* orb = reinterpret_cast<R*>(cv.take<char>(sizeof(R) * (size_t)npv * TS_ORB));
  R* ch = reinterpret_cast<R*>(cv.take<char>(sizeof(R) * (size_t)npv * npb * TS_CH));
  R* ldm = reinterpret_cast<R*>(cv.take<char>(sizeof(R) * (size_t)npv * npb * ng));
  double* kstat = cv.take<double>((size_t)npv * 2);
  ts_prepare_kernel<R><<<npv, TS_PREP_THREADS, 0, s>>>(k, t0, p, a, inc, e, w, istar, npv, npb, exptime0, t_ref,
                                                      t_absmax, orb, ch, kstat);
  // LD means at kmean: 3D table with the TS rule (kmin <= kmean <= max k), or the 2D table
  if (weights == nullptr) {
    dim3 g2(npv, (ng + TS_L2_ROWS - 1) / TS_L2_ROWS);
    ts_ldm2d_kernel<R><<<g2, 128, 0, s>>>(ldp, npb, nz, kstat, z_edges, ng, ldm);
  } else if constexpr (SPLIT) {
    launch_ldm_f32(ldp, npv, npb, nz, kstat, 1, weights, nk, ng, dk, kmin, kmax, z_edges, 1, kstat + npv, ldm, s);
  } else {
    launch_ldm_f64(ldp, npv, npb, nz, kstat, 1, weights, nk, ng, dk, kmin, kmax, z_edges, 1, kstat + npv, ldm, s);
  }
  const int ntiles = (npt + 127) / 128;
  const int max_bx = (ntiles + TS_WARPS - 1) / TS_WARPS;
  long long bx = (152LL * 16 + npv - 1) / npv;
  bx = bx < 1 ? 1 : (bx > max_bx ? max_bx : bx);
  dim3 fg((unsigned)bx, npv < 65535 ? npv : 65535, (npv + 65534) / 65535);
  ts_flux_kernel<R, SPLIT><<<fg, TS_WARPS * 32, 0, s>>>(times, reinterpret_cast<const float2*>(times_ff), npt,
                                                         t0, p, npv, npb, nsamples0, exptime0, orb, ch, ldm, ng, dg,
                                                         flux, ldflux);
  return check_launch("rr_ts");
}

extern "C" {

int rr_ts_f64(const double* times, int npt, const double* k, const double* t0, const double* p, const double* a,
              const double* inc, const double* e, const double* w, int npv, int npb, int nsamples0,
              double exptime0, const double* ldp, const double* istar, const double* weights, int nk, int ng,
              int nz, double dk, double kmin, double kmax, double dg, const double* z_edges, void* workspace,
              size_t workspace_bytes, double* flux, int ldflux, void* stream) {
  return ts_impl<double, false>(times, nullptr, 0.0, 0.0, npt, k, t0, p, a, inc, e, w, npv, npb, nsamples0,
                                exptime0, ldp, istar, weights, nk, ng, nz, dk, kmin, kmax, dg, z_edges, workspace,
                                workspace_bytes, flux, ldflux, stream);
}

int rr_ts_split(const float* times_ff, double t_ref, double t_absmax, int npt, const double* k, const double* t0,
                const double* p, const double* a, const double* inc, const double* e, const double* w, int npv,
                int npb, int nsamples0, double exptime0, const float* ldp, const float* istar,
                const float* weights, int nk, int ng, int nz, double dk, double kmin, double kmax, double dg,
                const double* z_edges, void* workspace, size_t workspace_bytes, float* flux, int ldflux,
                void* stream) {
  return ts_impl<float, true>(nullptr, times_ff, t_ref, t_absmax, npt, k, t0, p, a, inc, e, w, npv, npb, nsamples0,
                              exptime0, ldp, istar, weights, nk, ng, nz, dk, kmin, kmax, dg, z_edges, workspace,
                              workspace_bytes, flux, ldflux, stream);
}

}  // extern "C"
