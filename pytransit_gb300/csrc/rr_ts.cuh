// Transmission-spectroscopy flux for one 128-point tile of one parameter
// vector (tsmodel_serial's light-curve loop, pytransit/models/roadrunner/
// model_trspec.py:72-93), shared by the TS flux kernel (rr_ts.cu) and the
// persistent serving kernel (rr_full.cu).
//
// npb channels with their own radius ratio k_b share one orbit; the LD means
// are taken at kmean and the occulted area to first order in k:
//   area_b = afac_b A(kmean)                 z <= 1 - max k (fully inside)
//   area_b = A(kmean) + (k_b - kmean) dA/dk  otherwise,
// afac_b = k_b^2 / kmean^2.  For each channel the samples of a point touch a
// few consecutive rows j of the channel's LD-mean table L_b, and
//   sum_s I_b(g_s) area_b(s) = sum_j L_b[j] (afac_b win_j + wout_j + dk_b wd_j)
// with win/wout/wd the lerp weights of the samples times their area (inside
// or on the limb) and dA/dk.  So a tile is done in two phases:
//   1. one thread per point: the fold, the box test, and the weights of the
//      point's samples on at most TS_MW table rows, into shared memory;
//   2. warps over channels, each lane over 4 consecutive points: the table
//      rows against the weights, one 16-byte store per lane per channel row
//      (a tile without in-box points is the same loop storing the fill value).
// A point whose samples span more than TS_MW rows is done after the tile by
// one warp, lanes over its samples and then over the channels.
#pragma once
#include "rr_device.cuh"
#include "rr_internal.h"

namespace rr {

constexpr int TS_ORB = 32;    // per-pv record (R)
// record fields: c[0..9], [10] t1, [11] t4 (padded box), [12] kmean,
// [13] 1/(1+kmean), [14] 1 - max(k), [15] valid, [16] p_hi, [17] p_lo,
// [18] 1/p, [19] d0_hi, [20] d0_lo, [21] fast-test error bound, [22] wide flag,
// [23] stated maximum absolute flux error of the pv (split path)
constexpr int TS_CH = 4;      // per-channel record: afac, k - kmean, 1/istar, unused
constexpr int TS_MW = 8;      // LD-table rows a point keeps weights for
constexpr int TS_TILE = 128;  // points per tile

template <typename R>
struct TsSmem {
  R w[3][TS_MW][TS_TILE];     // win, wout, wd per row per point
  int jlo[TS_TILE];
  int nrow[TS_TILE];
  int wide[TS_TILE];          // points for the warp path
  int nwide;
  int flags;
  unsigned reach;             // ts_range: the range's tiles that reach a box copy
};

template <typename R>
struct TsArgs {
  const double* times;        // plain path: FP64 times
  const float2* times_ff;     // split path: FP32-pair times and tile summaries
  const double *t0, *p;       // plain path: the fold in FP64
  const R *orb, *ch, *ldm;    // [npv][TS_ORB], [npv][npb][TS_CH], [npv][npb][ng]
  R* flux;                    // [npv][npb][ldflux]
  long long ldflux;
  int npt, npb, ng, nsamples0;
  double exptime0, dg;
  const double* tiles64;      // plain path: FP64 tile summaries (rr_time_tiles_f64) for the tile cull, or null
};

// Phase-folded time of point pt (time from the nearest conjunction): FP32
// pairs with error-free transformations in the split path, the reference's
// FP64 fold (model_trspec.py:74-76) in the plain path.
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

// Tile cull of the split path: can any point of the tile (its time range
// from the tile summary) fall in a box copy of the pv?  The fast-test error
// bound widens the box.
__device__ __forceinline__ bool ts_tile_reaches_box(const float4 tm, const float* o) {
  const float d0h = o[19], p_hi = o[16], inv_p = o[18], err = o[21];
  const float smin = tm.x - d0h, smax = tm.y - d0h;
  const float flo = o[10] - err, fhi = o[11] + err;
  const float j0 = ceilf((smin - fhi) * inv_p);
  bool hit = false;
#pragma unroll
  for (int dj = -1; dj <= 1; ++dj) {
    const float jj = j0 + (float)dj;
    hit = hit || (fmaf(jj, p_hi, flo) <= smax && fmaf(jj, p_hi, fhi) >= smin);
  }
  return hit;
}

// 16-byte store of four consecutive values (two 16-byte stores for FP64).
__device__ __forceinline__ void ts_store4(float* dst, float a, float b, float c, float d) {
  __stcs(reinterpret_cast<float4*>(dst), make_float4(a, b, c, d));
}
__device__ __forceinline__ void ts_store4(double* dst, double a, double b, double c, double d) {
  __stcs(reinterpret_cast<double2*>(dst), make_double2(a, b));
  __stcs(reinterpret_cast<double2*>(dst) + 1, make_double2(c, d));
}

// The tile `tile` of parameter vector pv (record o, in shared or global
// memory), by every thread of the block (blockDim.x a multiple of 32, at
// least TS_TILE); every branch around a barrier is block-uniform.  A tile that
// uses S begins with a barrier, so consecutive calls may share S; the caller
// synchronises before it rewrites the record o.
template <typename R, bool SPLIT>
__device__ __forceinline__ void ts_tile(const TsArgs<R>& A, int pv, int tile, const R* o, TsSmem<R>& S,
                                        bool culled_by_caller = false) {
  const unsigned FULL = 0xffffffffu;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, nwarps = blockDim.x >> 5;
  const int npt = A.npt, npb = A.npb, ng = A.ng;
  const bool valid = o[15] != R(0);
  const int pt0 = tile * TS_TILE;
  R* fpv = A.flux + (size_t)pv * npb * A.ldflux;
  // --- phase 1: one thread per point -------------------------------------
  bool any = false;
  int flags = 0;   // bit 0: in-box points in the tile, bit 1: a point with more than two rows
  if (valid) {
    bool reach = true;
    if constexpr (SPLIT) {
      static_assert(sizeof(R) == 4, "the split path keeps FP32 records");
      if (!culled_by_caller && !(o[22] != R(0))) {
        const float4* meta = reinterpret_cast<const float4*>(reinterpret_cast<const float*>(A.times_ff) +
                                                             time_meta_offset(npt));
        reach = ts_tile_reaches_box(__ldg(meta + tile), reinterpret_cast<const float*>(o));
      }
    }
    if (reach) {
      __syncthreads();   // every warp is done with S for the previous tile
      if (tid == 0) {
        S.nwide = 0;
        S.flags = 0;
      }
      __syncthreads();
      int nrow = 0, jlo = 0;
      const int pt = pt0 + tid;
      if (tid < TS_TILE) {
        // rows 0 and 1 are read for every point by the two-row path of phase 2
#pragma unroll
        for (int k = 0; k < 3; ++k) S.w[k][0][tid] = S.w[k][1][tid] = R(0);
      }
      if (tid < TS_TILE && pt < npt) {
        const double tz = SPLIT ? 0.0 : A.t0[pv], pp = SPLIT ? 0.0 : A.p[pv];
        const R tc = ts_fold<R, SPLIT>(pt, A.times, A.times_ff, tz, pp, o);
        if (o[10] <= tc && tc <= o[11]) {
          R cc[10];
#pragma unroll
          for (int i = 0; i < 10; ++i) cc[i] = o[i];
          const R kmean = o[12], inv1pk = o[13], inner_lim = o[14];
          const R inv_dg = R(1) / (R)A.dg;
          const R ex = (R)A.exptime0, inv_ns = R(1) / (R)A.nsamples0;
          const int ns = A.nsamples0;
          // pass 1: the rows the samples touch
          int lo = 0x7fffffff, hi = -1;
          for (int s = 0; s < ns; ++s) {
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
          const int nwin = hi >= 0 ? hi - lo + 1 : 0;
          bool wide = nwin > TS_MW;
          bool act = false;
          // pass 2: the row weights, accumulated in the point's own column of S.w
          // (a row outside the window of pass 1, possible only through a
          // different rounding of z, sends the point to the warp path)
          if (nwin > 0 && !wide) {
            for (int j = 2; j < nwin; ++j) S.w[0][j][tid] = S.w[1][j][tid] = S.w[2][j][tid] = R(0);
            for (int s = 0; s < ns; ++s) {
              const R t = tc + ex * ((R(s) + R(0.5)) * inv_ns - R(0.5));
              R a, dadk, fr;
              int gi;
              bool inner;
              if (!ts_sample<R>(t, cc, kmean, inv1pk, inv_dg, ng, inner_lim, a, dadk, gi, fr, inner)) continue;
              const int j0 = gi - lo;
              if (j0 < 0 || j0 + 1 >= nwin) {
                wide = true;
                break;
              }
              act = true;
              const R w0 = R(1) - fr;
              if (inner) {
                S.w[0][j0][tid] += w0 * a;
                S.w[0][j0 + 1][tid] += fr * a;
              } else {
                S.w[1][j0][tid] += w0 * a;
                S.w[1][j0 + 1][tid] += fr * a;
                S.w[2][j0][tid] += w0 * dadk;
                S.w[2][j0 + 1][tid] += fr * dadk;
              }
            }
          }
          if (wide) {
            S.wide[atomicAdd(&S.nwide, 1)] = pt;
            act = false;
          }
          if (act) {
            nrow = nwin;
            jlo = lo;
          }
          if (act || wide) atomicOr(&S.flags, (act ? 1 : 0) | (wide ? 1 : 0) | (nwin > 2 && act ? 2 : 0));
        }
      }
      if (tid < TS_TILE) {
        S.jlo[tid] = jlo;
        S.nrow[tid] = nrow;
      }
      __syncthreads();
      flags = S.flags;
      any = flags != 0;
    }
  }
  // --- phase 2: warps over channels, lanes over 4 consecutive points --------
  const int p0 = pt0 + 4 * lane;
  const bool vec = ((A.ldflux & 3) == 0) && ((reinterpret_cast<uintptr_t>(A.flux) & 15) == 0) && p0 + 3 < npt;
  if (!any) {
    const R fill = valid ? R(1) : R(CUDART_NAN);
    for (int b = warp; b < npb; b += nwarps) {
      R* dst = fpv + (size_t)b * A.ldflux + p0;
      if (vec) {
        ts_store4(dst, fill, fill, fill, fill);
      } else {
        for (int q = 0; q < 4; ++q)
          if (p0 + q < npt) dst[q] = fill;
      }
    }
    return;
  }
  const int4 nr4 = *reinterpret_cast<const int4*>(S.nrow + 4 * lane);
  const int4 jl4 = *reinterpret_cast<const int4*>(S.jlo + 4 * lane);
  const int nr[4] = {nr4.x, nr4.y, nr4.z, nr4.w};
  const int jl[4] = {jl4.x, jl4.y, jl4.z, jl4.w};
  const R inv_ns = R(1) / (R)A.nsamples0;
  const R* ldm_pv = A.ldm + (size_t)pv * npb * ng;
  const R* ch_pv = A.ch + (size_t)pv * npb * TS_CH;
  if (!(flags & 2)) {
    // Every in-box point's samples touch two rows (always so with one sample
    // per point): the lane's 4 points' 6 weights stay in registers, and two
    // channels are evaluated per iteration so that their loads overlap.
    R wgt[3][2][4];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int j = 0; j < 2; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) wgt[k][j][q] = S.w[k][j][4 * lane + q];
    for (int b = warp; b < npb; b += 2 * nwarps) {
      const int bc[2] = {b, min(b + nwarps, npb - 1)};
      R cf[2][3], l0[2][4], l1[2][4];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const R* cr = ch_pv + (size_t)bc[u] * TS_CH;
        cf[u][0] = __ldg(cr);
        cf[u][1] = __ldg(cr + 1);
        cf[u][2] = __ldg(cr + 2) * inv_ns;
        const R* Lb = ldm_pv + (size_t)bc[u] * ng;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          l0[u][q] = nr[q] > 0 ? __ldg(Lb + jl[q]) : R(0);
          l1[u][q] = nr[q] > 0 ? __ldg(Lb + jl[q] + 1) : R(0);
        }
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        if (u == 1 && b + nwarps >= npb) break;
        R v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const R fi = l0[u][q] * wgt[0][0][q] + l1[u][q] * wgt[0][1][q];
          const R fo = l0[u][q] * wgt[1][0][q] + l1[u][q] * wgt[1][1][q];
          const R fd = l0[u][q] * wgt[2][0][q] + l1[u][q] * wgt[2][1][q];
          v[q] = nr[q] > 0 ? R(1) - (cf[u][0] * fi + fo + cf[u][1] * fd) * cf[u][2] : R(1);   // out of box: exactly 1
        }
        R* dst = fpv + (size_t)bc[u] * A.ldflux + p0;
        if (vec) {
          ts_store4(dst, v[0], v[1], v[2], v[3]);
        } else {
          for (int q = 0; q < 4; ++q)
            if (p0 + q < npt) dst[q] = v[q];
        }
      }
    }
  } else {
    const int mrow = max(max(nr[0], nr[1]), max(nr[2], nr[3]));
    for (int b = warp; b < npb; b += nwarps) {
      const R* cr = ch_pv + (size_t)b * TS_CH;
      const R afac = __ldg(cr), dkb = __ldg(cr + 1), scale = __ldg(cr + 2) * inv_ns;
      const R* Lb = ldm_pv + (size_t)b * ng;
      R acc[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[q] = R(0);
      for (int j = 0; j < mrow; ++j) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          if (j < nr[q]) {
            const R l = __ldg(Lb + jl[q] + j);
            acc[q] += l * (afac * S.w[0][j][4 * lane + q] + S.w[1][j][4 * lane + q] +
                           dkb * S.w[2][j][4 * lane + q]);
          }
        }
      }
      R v[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = nr[q] > 0 ? R(1) - acc[q] * scale : R(1);   // out of box: exactly 1
      R* dst = fpv + (size_t)b * A.ldflux + p0;
      if (vec) {
        ts_store4(dst, v[0], v[1], v[2], v[3]);
      } else {
        for (int q = 0; q < 4; ++q)
          if (p0 + q < npt) dst[q] = v[q];
      }
    }
  }
  // --- points whose samples span more than TS_MW rows: a warp per point ----
  __syncthreads();   // phase 2 wrote 1.0 for them; the barrier orders the overwrite
  const int nw = S.nwide;
  if (nw == 0) return;
  R cc[10];
#pragma unroll
  for (int i = 0; i < 10; ++i) cc[i] = o[i];
  const R kmean = o[12], inv1pk = o[13], inner_lim = o[14];
  const R inv_dg = R(1) / (R)A.dg;
  const R ex = (R)A.exptime0;
  const int ns = A.nsamples0;
  const double tz = SPLIT ? 0.0 : A.t0[pv], pp = SPLIT ? 0.0 : A.p[pv];
  for (int iw = warp; iw < nw; iw += nwarps) {
    const int ptw = S.wide[iw];
    const R tcw = ts_fold<R, SPLIT>(ptw, A.times, A.times_ff, tz, pp, o);
    for (int s0 = 0; s0 < ns; s0 += 32) {
      const int ns_here = min(32, ns - s0);
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
        const R* cr = ch_pv + (size_t)bb * TS_CH;
        const R afac = cr[0], dkb = cr[1];
        const R* Lb = ldm_pv + (size_t)bb * ng;
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
          R* dst = fpv + (size_t)b * A.ldflux + ptw;
          // samples beyond the first 32 add to the value already stored
          const R prev = (s0 == 0) ? R(1) : *dst;
          *dst = prev - acc * cr[2] * inv_ns;
        }
      }
      __syncwarp();
    }
  }
}

// Fill of the tiles [ta, tb) of every channel row of pv with `fill`, row
// by row: each warp writes one row's segment as one contiguous run (16-byte
// stores), so that the output reaches DRAM in long runs rather than in
// 512-byte pieces 200 rows apart.
template <typename R>
__device__ __forceinline__ void ts_fill_rows(const TsArgs<R>& A, int pv, int ta, int tb, R fill) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  const int p0 = ta * TS_TILE, p1 = min(A.npt, tb * TS_TILE);
  R* fpv = A.flux + (size_t)pv * A.npb * A.ldflux;
  const bool vec = ((A.ldflux & 3) == 0) && ((reinterpret_cast<uintptr_t>(A.flux) & 15) == 0);
  const int n4 = vec ? (p1 - p0) >> 2 : 0;   // whole groups of 4 from p0 (a multiple of 4)
  for (int b = warp; b < A.npb; b += nwarps) {
    R* row = fpv + (size_t)b * A.ldflux;
    for (int i = lane; i < n4; i += 32) ts_store4(row + p0 + 4 * i, fill, fill, fill, fill);
    for (int pt = p0 + 4 * n4 + lane; pt < p1; pt += 32) row[pt] = fill;
  }
}

// The tiles [tb0, tb1) of pv (tb1 - tb0 <= 32), by the whole block: one warp
// tests the tiles against the box copies (split path: from the tile
// summaries), the runs of tiles that reach none are filled row by row, and
// the others go through ts_tile.  The plain path has no tile summaries:
// every tile of a valid pv goes through ts_tile.
template <typename R, bool SPLIT>
__device__ __forceinline__ void ts_range(const TsArgs<R>& A, int pv, int tb0, int tb1, const R* o, TsSmem<R>& S) {
  const int n = tb1 - tb0;
  const bool valid = o[15] != R(0);
  if (!valid) {
    ts_fill_rows<R>(A, pv, tb0, tb1, R(CUDART_NAN));
    return;
  }
  unsigned reach = n >= 32 ? 0xffffffffu : (1u << n) - 1u;
  if constexpr (!SPLIT) {
    // The plain path with tile summaries: the reference's FP64 fold
    // (model_trspec.py:74-76) is non-decreasing in t with its own rounding, so
    // a tile whose earliest and latest times share an epoch, and whose two
    // ends' tc miss the box, holds 1.0 at every point (the same bits as the
    // per-point path).
    if (A.tiles64) {
      __syncthreads();                 // S.reach of a previous range is consumed
      if ((threadIdx.x >> 5) == 0) {
        const int lane = threadIdx.x & 31;
        bool hit = false;
        if (lane < n) {
          const double* tl = A.tiles64 + 4 * (size_t)(tb0 + lane);
          const double tz = A.t0[pv], pp = A.p[pv];
          const double e0 = floor(__ddiv_rn(__dadd_rn(__dsub_rn(tl[0], tz), __dmul_rn(0.5, pp)), pp));
          const double e1 = floor(__ddiv_rn(__dadd_rn(__dsub_rn(tl[1], tz), __dmul_rn(0.5, pp)), pp));
          hit = true;
          if (e0 == e1) {
            const double c = __dadd_rn(tz, __dmul_rn(e0, pp));
            hit = !(__dsub_rn(tl[1], c) < (double)o[10] || __dsub_rn(tl[0], c) > (double)o[11]);
          }
        }
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) S.reach = m;
      }
      __syncthreads();
      reach = S.reach;
    }
  }
  if constexpr (SPLIT) {
    if (!(o[22] != R(0))) {
      __syncthreads();                 // S.reach of a previous range is consumed
      if ((threadIdx.x >> 5) == 0) {
        const int lane = threadIdx.x & 31;
        const float4* meta = reinterpret_cast<const float4*>(reinterpret_cast<const float*>(A.times_ff) +
                                                             time_meta_offset(A.npt));
        const bool hit = lane < n && ts_tile_reaches_box(__ldg(meta + tb0 + lane), reinterpret_cast<const float*>(o));
        const unsigned m = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) S.reach = m;
      }
      __syncthreads();
      reach = S.reach;
    }
  }
  // runs of tiles that reach no box copy, row by row
  const unsigned all = n >= 32 ? 0xffffffffu : (1u << n) - 1u;
  unsigned rest = ~reach & all;
  while (rest) {
    const int a = __ffs(rest) - 1;
    const unsigned above = ~((2u << a) - 1u);          // bits above a (0 for a = 31)
    const unsigned stop = reach & above & all;
    const int b = stop ? __ffs(stop) - 1 : n;
    ts_fill_rows<R>(A, pv, tb0 + a, tb0 + b, R(1));
    rest &= b >= 32 ? 0u : ~((1u << b) - 1u);
  }
  for (unsigned m = reach; m; m &= m - 1u) ts_tile<R, SPLIT>(A, pv, tb0 + __ffs(m) - 1, o, S, true);
}

}  // namespace rr
