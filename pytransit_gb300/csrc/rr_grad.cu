// Gaussian log-likelihood of the RoadRunner model and its adjoint:
//   lnL[pv] = sum_i -log(sigma_i) - log(2 pi)/2 - ((o_i - m_i(theta_pv)) / sigma_i)^2 / 2
// (pytransit/lpf/loglikelihood/wnloglikelihood.py:23-35; lpf.py:51-66), fused
// with the model so the flux is never stored, and d lnL / d theta for
// theta = (k, t0, p, a, i, e, w, ldc), recomputing z, the table interpolation
// and the area per sample in the backward pass.
//
// The derivative is that of the discretised model: the k-interpolation of the
// weight table, the g-interpolation of the LD means, the kite area, the
// coefficient dependence of the LD profile and of its disk integral, and the
// orbit's Taylor coefficients (forward-mode duals through the jet solve).  The
// bounding box and the epoch count are piecewise constant and contribute no
// derivative.  Out-of-box points (F = 1 exactly) only enter through the
// pv-independent constant sum_i -log sigma_i - log(2 pi)/2 - (o_i - 1)^2/(2 sigma_i^2).
#include <cmath>

#include "rr_device.cuh"
#include "rr_dual.cuh"
#include "rr_internal.h"

namespace rr {

constexpr int MAX_GRAD_PAR = 4;    // LD coefficients per passband in the adjoint
constexpr int MAX_NGRAD = 64;      // nkc + nep + 5 + npb * npar
constexpr int GLC_SMEM = 64;       // light-curve records staged in shared memory (split)

// Slots of one point's gradient contribution: destinations vary per point.
enum GSlot { GS_LNL = 0, GS_KK, GS_KW, GS_T0, GS_P, GS_A, GS_I, GS_E, GS_W, GS_C0, GS_NSLOT = GS_C0 + MAX_GRAD_PAR };

// ---------------------------------------------------------------------------
// Prologue 1: derivatives of the orbit's Taylor coefficients, one thread per
// pv: dc[pv][j][m] = d c_m / d theta_j, theta = (p, a, i, e, w).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void grad_orbit_kernel(const double* __restrict__ p, const double* __restrict__ a,
                                  const double* __restrict__ inc, const double* __restrict__ e,
                                  const double* __restrict__ w, int npv, R* __restrict__ dc) {
  const int pv = blockIdx.x * blockDim.x + threadIdx.x;
  if (pv >= npv) return;
  D5 c[10];
  solve2d_conj_dual(p[pv], a[pv], inc[pv], e[pv], w[pv], c);
  R* o = dc + (size_t)pv * 50;
  for (int j = 0; j < 5; ++j)
    for (int m = 0; m < 10; ++m) o[j * 10 + m] = (R)c[m].d[j];
}

// ---------------------------------------------------------------------------
// Prologue 2: LD-table derivatives, one block per (pv, pb):
//   dL/dk[g]   = (W[ik+1] @ ldp - W[ik] @ ldp)[g] / dk   (3D table), or a
//                central difference of the 2D table at k +- h;
//   dL/dc_j[g] = Wk @ (d ldp / d c_j), Wk the table the forward pass uses;
//   d istar / d c_j analytic, or the 200-point trapezoid of z dI/dc_j.
// tab layout per (pv, pb): [dL/dk (ng)][dL/dc_0 (ng)]...[dL/dc_{npar-1} (ng)],
// dis layout: [d istar/dc_j] (npar).
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(128)
grad_ld_kernel(int law, const double* __restrict__ ldc, int npb, int npar, const double* __restrict__ mu,
               int nz, const R* __restrict__ ldp, const double* __restrict__ kw, int kw_stride,
               const R* __restrict__ W, int nk, int ng, double dk, double kmin, double kmax,
               const double* __restrict__ ze, R* __restrict__ tab, R* __restrict__ dis) {
  __shared__ R l[64];
  __shared__ R dl[MAX_GRAD_PAR][64];
  __shared__ R pvs[16];
  const int pv = blockIdx.x, pb = blockIdx.y;
  const size_t ppb = (size_t)pv * npb + pb;
  if (threadIdx.x < npar) pvs[threadIdx.x] = (R)ldc[ppb * npar + threadIdx.x];
  __syncthreads();
  for (int z = threadIdx.x; z < nz; z += blockDim.x) {
    l[z] = ldp[ppb * nz + z];
    for (int j = 0; j < npar; ++j) dl[j][z] = ld_dvalue<R>(law, (R)mu[z], pvs, npar, j);
  }
  if (threadIdx.x < npar) {
    const int j = threadIdx.x;
    R d;
    if (!ld_dintegral<R>(law, pvs, j, d)) {
      const int NT = 200;
      R s = R(0), z0 = R(0), y0 = R(0);
      for (int i = 0; i < NT; ++i) {
        R m = R(NT - 1 - i) / R(NT - 1);
        R z = sqrt(R(1) - m * m);
        R y = z * ld_dvalue<R>(law, m, pvs, npar, j);
        if (i > 0) s += (z - z0) * (y + y0) / R(2);
        z0 = z;
        y0 = y;
      }
      d = R(2.0 * PI) * s;
    }
    dis[ppb * npar + j] = d;
  }
  __syncthreads();
  const double k = kw[(size_t)pv * kw_stride];
  int ik = -1;
  double ak = 0.0;
  if (kmin <= k && k <= kmax) {
    ik = (int)floor((k - kmin) / dk);
    ak = (k - kmin - ik * dk) / dk;
    if (ik + 1 >= nk || ik < 0) ik = -1;
  }
  R* out = tab + ppb * (size_t)(1 + npar) * ng;
  const double gstep = (1.0 - 1e-7) / (double)(ng - 1);
  for (int g = threadIdx.x; g < ng; g += blockDim.x) {
    if (ik >= 0) {
      const R* w0 = W + ((size_t)ik * ng + g) * nz;
      const R* w1 = w0 + (size_t)ng * nz;
      R d0 = R(0), d1 = R(0);
      R c0[MAX_GRAD_PAR] = {}, c1[MAX_GRAD_PAR] = {};
      for (int z = 0; z < nz; ++z) {
        const R a0 = __ldg(w0 + z), a1 = __ldg(w1 + z);
        d0 += a0 * l[z];
        d1 += a1 * l[z];
        for (int j = 0; j < npar; ++j) {
          c0[j] += a0 * dl[j][z];
          c1[j] += a1 * dl[j][z];
        }
      }
      out[g] = (R)(((double)d1 - (double)d0) / dk);
      for (int j = 0; j < npar; ++j) out[(size_t)(1 + j) * ng + g] = (R(1) - (R)ak) * c0[j] + (R)ak * c1[j];
    } else {
      // 2D table at k (and at k +- h for the k derivative), FP64 rows
      double gg = (g == ng - 1) ? (1.0 - 1e-7) : (double)g * gstep;
      const double h = 1e-6 * fmax(k, 1e-3);
      double res[3][1 + MAX_GRAD_PAR];
      for (int v = 0; v < 3; ++v) {
        const double kv = k + (v - 1) * h;
        const double bb = gg * (1.0 + kv);
        double a0 = cci_acos(ze[0], kv, bb), s = a0;
        double acc[1 + MAX_GRAD_PAR];
        acc[0] = a0 * (double)l[0];
        for (int j = 0; j < npar; ++j) acc[1 + j] = a0 * (double)dl[j][0];
        for (int z = 1; z < nz; ++z) {
          const double a1 = cci_acos(ze[z], kv, bb), wz = a1 - a0;
          a0 = a1;
          s += wz;
          acc[0] += wz * (double)l[z];
          for (int j = 0; j < npar; ++j) acc[1 + j] += wz * (double)dl[j][z];
        }
        for (int j = 0; j <= npar; ++j) res[v][j] = acc[j] / s;
      }
      out[g] = (R)((res[2][0] - res[0][0]) / (2.0 * h));
      for (int j = 0; j < npar; ++j) out[(size_t)(1 + j) * ng + g] = (R)res[1][1 + j];
    }
  }
}

// ---------------------------------------------------------------------------
// Observations: dobs[i] = o_i - 1 and isig2[i] = 1/sigma_lc^2 in R, and the
// pv-independent constant of lnL in per-block parts (FP64, fixed order), one
// block per OBS_CHUNK points.
// ---------------------------------------------------------------------------
constexpr int OBS_THREADS = 128;
constexpr int OBS_CHUNK = OBS_THREADS * 4;

template <typename R>
__global__ void __launch_bounds__(OBS_THREADS) obs_kernel(const double* __restrict__ obs,
                                                          const double* __restrict__ sigma,
                                                          const int32_t* __restrict__ lcids, int npt,
                                                          R* __restrict__ dobs, R* __restrict__ isig2,
                                                          double* __restrict__ cpart) {
  __shared__ double red[OBS_THREADS / 32];
  double acc = 0.0;
  const double hl2pi = 0.5 * log(2.0 * PI);
  const int i0 = blockIdx.x * OBS_CHUNK, i1 = min(npt, i0 + OBS_CHUNK);
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const double s = sigma[lcids[i]];
    const double d = obs[i] - 1.0;
    dobs[i] = (R)d;
    isig2[i] = (R)(1.0 / (s * s));
    acc += -log(s) - hl2pi - 0.5 * (d / s) * (d / s);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sm = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) sm += red[i];
    cpart[blockIdx.x] = sm;
  }
}

// ---------------------------------------------------------------------------
// Main kernel: blocks over (chunk of points, pv), each thread a few points.
// For in-box points: per sample the sky position and its derivatives (Horner
// on c and on dc), z, the area and its partials, the interpolated mean
// intensity and its partials; per point D = sum_s I A / (ns istar); lnL gets
// -(do + D/2) D / sigma^2, the gradient -(r / sigma^2) dD/dtheta with
// r = do + D.  Block sums go to partials[pv][block][1 + ngrad] (FP64), summed
// per pv in block order by lnlike_reduce_kernel: no step depends on timing.
// ---------------------------------------------------------------------------
template <typename R>
struct GradArgs {
  // data
  const double* times;          // FP64 path
  const float2* times_ff;       // split path
  const int32_t *lcids, *pbids, *epids, *nsamples;
  const double* exptimes;
  const R *dobs, *isig2;
  // parameters (FP64 path reads them directly)
  const double *k, *t0, *p, *istar64;
  int nkc, ldt0, nep;
  // prologue tables
  const double* orb64;
  const float *orb32, *lc32;
  const R *ldm, *dc, *tab, *dis;
  int npt, npv, npb, nlc, ng, npar, ngrad;
  double dg;
  int grad;
  double* partials;
};

__device__ __forceinline__ int grad_col(int slot, int nkc, int nep, int npar, int pb, int ep, int j) {
  switch (slot) {
    case GS_KK: return (nkc == 1) ? 0 : pb;
    case GS_KW: return 0;
    case GS_T0: return nkc + ep;
    case GS_P: case GS_A: case GS_I: case GS_E: case GS_W: return nkc + nep + (slot - GS_P);
    default: return nkc + nep + 5 + pb * npar + j;
  }
}

// Launch shape of the likelihood kernel: blocks of LNL_THREADS threads over
// LNL_CHUNK consecutive points of one pv, LNL_PPT points per thread.
constexpr int LNL_THREADS = 128;
constexpr int LNL_PPT = 8;
constexpr int LNL_CHUNK = LNL_THREADS * LNL_PPT;
constexpr int LNL_NW = LNL_THREADS / 32;

// Adds one point's terms to the slot accumulators acc (the lnL term and, with
// GRAD, the gradient terms of GS_KK ... GS_C0 + npar - 1); nothing for a point
// out of the box.  Two passes over the samples: the first gives the point's
// deficit D and with it the residual weight -(r / sigma^2) / (ns istar); the
// second recomputes each sample and adds its derivative terms, already
// scaled by that weight, straight into acc (no per-point sums are kept).
template <typename R, bool SPLIT, bool GRAD>
__device__ __forceinline__ void lnlike_point(const GradArgs<R>& A, int pv, int pt, int lc, const float* lcs,
                                             bool lc_smem, const R* orbc, const R* dcs, R* acc) {
  const int pb = A.pbids[lc], ep = A.epids[lc];
  bool inbox;
  R tc, nep_count;
  if (SPLIT) {
    const float* LCR = lc_smem ? lcs + lc * LC32 : A.lc32 + ((size_t)pv * A.nlc + lc) * LC32;
    const float* o = A.orb32 + (size_t)pv * ORB32;
    const float p_hi = o[10], p_lo = o[11], inv_p = o[12];
    const float2 tt = A.times_ff[pt];
    const float d0h = LCR[LC_D0H], d0l = LCR[LC_D0L];
    float n = floorf(fmaf(tt.x - d0h, inv_p, 0.5f));
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
    inbox = (LCR[LC_LO] <= t && t <= LCR[LC_HI]);
    tc = (R)t;
    nep_count = (R)n;
  } else {
    const double t = A.times[pt];
    const double t0 = A.t0[(size_t)pv * A.ldt0 + ep];
    const double p = A.p[pv];
    const double epoch = floor(__ddiv_rn(__dadd_rn(__dsub_rn(t, t0), __dmul_rn(0.5, p)), p));
    const double tcd = __dsub_rn(t, __dadd_rn(t0, __dmul_rn(epoch, p)));
    const double pad = __dadd_rn(0.003, A.exptimes[lc]);
    const double* o = A.orb64 + (size_t)pv * ORB64;
    inbox = (__dsub_rn(o[10], pad) <= tcd && tcd <= __dadd_rn(o[11], pad));
    tc = (R)tcd;
    nep_count = (R)epoch;
  }
  if (!inbox) return;
  R kk, inv_is, ex, inv_ns;
  int ns;
  if (SPLIT) {
    const float* LCR = lc_smem ? lcs + lc * LC32 : A.lc32 + ((size_t)pv * A.nlc + lc) * LC32;
    kk = (R)LCR[LC_K];
    inv_is = (R)LCR[LC_INVIS];
    ex = (R)LCR[LC_EXPT];
    inv_ns = (R)LCR[LC_INVNS];
    ns = __float_as_int(LCR[LC_NS]);
  } else {
    kk = (R)A.k[(size_t)pv * A.nkc + (A.nkc == A.npb ? pb : 0)];
    inv_is = R(1) / (R)A.istar64[(size_t)pv * A.npb + pb];
    ex = (R)A.exptimes[lc];
    ns = A.nsamples[lc];
    inv_ns = R(1) / (R)ns;
  }
  const R inv1pk = R(1) / (R(1) + kk);
  const R inv_dg = R(1) / (R)A.dg;
  const size_t ppb = (size_t)pv * A.npb + pb;
  const R* L = A.ldm + ppb * A.ng;
  // pass 1: the deficit D = sum_s I A / (ns istar)
  R SQ = R(0);
  for (int s = 0; s < ns; ++s) {
    const R t = tc + ex * ((R(s) + R(0.5)) * inv_ns - R(0.5));
    R x = orbc[4], y = orbc[9];
    for (int m = 3; m >= 0; --m) {
      x = x * t + orbc[m];
      y = y * t + orbc[5 + m];
    }
    const R z = sqrt(x * x + y * y);
    if (!(z < R(1) + kk)) continue;  // A = 0 and I A = 0 beyond first contact
    const R gg = z * inv1pk * inv_dg;
    const int i = min(max((int)gg, 0), A.ng - 2);
    const R fr = gg - (R)i;
    const R l0 = L[i], l1 = L[i + 1];
    R kap;
    SQ += (l0 + fr * (l1 - l0)) * ccia_star<R>(kk, z, kap);
  }
  const R sc = inv_is * inv_ns;
  const R D = SQ * sc;
  const R do_ = A.dobs[pt], w = A.isig2[pt];
  acc[GS_LNL] += -(do_ + R(0.5) * D) * D * w;
  if constexpr (GRAD) {
    const R gsc = -(do_ + D) * w * sc;    // -(r / sigma^2) / (ns istar)
    const R* T = A.tab + ppb * (size_t)(1 + A.npar) * A.ng;
    // pass 2: the derivative terms of every sample, times gsc
    for (int s = 0; s < ns; ++s) {
      const R t = tc + ex * ((R(s) + R(0.5)) * inv_ns - R(0.5));
      R x = orbc[4], y = orbc[9], xd = R(4) * orbc[4], yd = R(4) * orbc[9];
      for (int m = 3; m >= 0; --m) {
        x = x * t + orbc[m];
        y = y * t + orbc[5 + m];
        if (m >= 1) {
          xd = xd * t + R(m) * orbc[m];
          yd = yd * t + R(m) * orbc[5 + m];
        }
      }
      const R z = sqrt(x * x + y * y);
      if (!(z < R(1) + kk)) continue;
      const R g = z * inv1pk;
      const R gg = g * inv_dg;
      const int i = min(max((int)gg, 0), A.ng - 2);
      const R fr = gg - (R)i;
      const R l0 = L[i], l1 = L[i + 1];
      const R ip = l0 + fr * (l1 - l0);
      R dadk, dadz;
      const R ar = ccia_star_grad<R>(kk, z, dadk, dadz);
      const R gar = gsc * ar;
      const R iz = R(1) / z;
      const R dzdt = (x * xd + y * yd) * iz;
      const R dIdg = (l1 - l0) * inv_dg;
      const R gdz = gsc * (dIdg * inv1pk * ar + ip * dadz);   // gsc dQ/dz
      acc[GS_KK] += gsc * (-dIdg * g * inv1pk * ar + ip * dadk);
      acc[GS_KW] += (T[i] + fr * (T[i + 1] - T[i])) * gar;
#pragma unroll
      for (int j = 0; j < MAX_GRAD_PAR; ++j) {
        if (j < A.npar) {
          const R* Tj = T + (size_t)(1 + j) * A.ng;
          acc[GS_C0 + j] += (Tj[i] + fr * (Tj[i + 1] - Tj[i])) * gar;
        }
      }
      // dz/dtheta: orbit coefficients (p, a, i, e, w) and the time shift of t0, p
      acc[GS_T0] += gdz * (-dzdt);
#pragma unroll
      for (int jj = 0; jj < 5; ++jj) {
        const R* d = dcs + jj * 10;
        R dx = d[4], dy = d[9];
        for (int m = 3; m >= 0; --m) {
          dx = dx * t + d[m];
          dy = dy * t + d[5 + m];
        }
        R dz = (x * dx + y * dy) * iz;
        if (jj == 0) dz += dzdt * (-nep_count);
        acc[GS_P + jj] += gdz * dz;
      }
    }
    // the disk integral's dependence on the LD coefficients
    const R* dI = A.dis + ppb * A.npar;
#pragma unroll
    for (int j = 0; j < MAX_GRAD_PAR; ++j)
      if (j < A.npar) acc[GS_C0 + j] += (do_ + D) * w * D * inv_is * dI[j];
  }
}

// Adds the accumulators of the lanes in `pending` to the warp's row of
// shared FP64 sums, one group of lanes sharing a light curve at a time
// (lowest lane first), each slot by the same shuffle tree; then clears them.
// Every step is in a fixed order, so the sums are reproducible bit for bit.
template <typename R, int NS>
__device__ __forceinline__ void lnlike_flush(const GradArgs<R>& A, R* acc, int key, bool pending, double* row) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int nsl = NS > 1 ? GS_C0 + A.npar : 1;
  unsigned pend = __ballot_sync(FULL, pending);
  while (pend) {
    const int leader = __ffs(pend) - 1;
    const int kl = __shfl_sync(FULL, key, leader);
    const unsigned mem = __ballot_sync(FULL, pending && key == kl) & pend;
    const bool in = (mem >> lane) & 1u;
    const int pb = A.pbids[kl], ep = A.epids[kl];
#pragma unroll
    for (int s = 0; s < NS; ++s) {
      if (s >= nsl) break;
      const int col = (s == GS_LNL) ? -1 : grad_col(s, A.nkc, A.nep, A.npar, pb, ep, s - GS_C0);
      double tot;
      if constexpr (sizeof(R) == 4) {
        // FP32 (hi, lo) pairs summed with error-free two-sums: as accurate as
        // an FP64 tree without the FP64 pipe (1/64 rate)
        float hi = in ? acc[s] : 0.0f, lo = 0.0f;
        for (int o = 16; o > 0; o >>= 1) {
          const float h2 = __shfl_down_sync(FULL, hi, o), l2 = __shfl_down_sync(FULL, lo, o);
          float sh, se;
          two_sum(hi, h2, sh, se);
          lo = lo + l2 + se;
          hi = sh;
        }
        tot = (double)hi + (double)lo;
      } else {
        double vv = in ? (double)acc[s] : 0.0;
        for (int o = 16; o > 0; o >>= 1) vv += __shfl_down_sync(FULL, vv, o);
        tot = vv;
      }
      if (lane == 0) row[col + 1] += tot;
    }
    if (in) {
#pragma unroll
      for (int s = 0; s < NS; ++s) acc[s] = R(0);
    }
    pend &= ~mem;
  }
}

// One block: LNL_CHUNK consecutive points of pv.  Each thread sums its points'
// terms in registers while they share a light curve (the gradient columns
// depend on its passband and epoch), flushing to its warp's row of shared
// sums when the light curve changes and at the end; the block writes the sum
// of the warps' rows, in warp order, to its slot of partials.
template <typename R, bool SPLIT, bool GRAD>
__global__ void __launch_bounds__(LNL_THREADS, sizeof(R) == 4 ? 4 : 2) lnlike_kernel(GradArgs<R> A) {
  constexpr int NS = GRAD ? GS_NSLOT : 1;
  __shared__ double wred[LNL_NW][1 + MAX_NGRAD];
  __shared__ __align__(16) float lcs[SPLIT ? GLC_SMEM * LC32 : 1];
  __shared__ R orbc[10];
  __shared__ R dcs[50];
  const int pv = blockIdx.y;
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < LNL_NW * (1 + MAX_NGRAD); i += blockDim.x) (&wred[0][0])[i] = 0.0;
  if (tid < 10)
    orbc[tid] = SPLIT ? (R)A.orb32[(size_t)pv * ORB32 + tid] : (R)A.orb64[(size_t)pv * ORB64 + tid];
  if (GRAD && tid < 50) dcs[tid] = A.dc[(size_t)pv * 50 + tid];
  const bool lc_smem = SPLIT && A.nlc <= GLC_SMEM;
  if (lc_smem)
    for (int i = tid; i < A.nlc * LC32; i += blockDim.x) lcs[i] = A.lc32[(size_t)pv * A.nlc * LC32 + i];
  __syncthreads();
  const bool valid = SPLIT ? (__float_as_int(A.orb32[(size_t)pv * ORB32 + 14]) & FLAG_VALID)
                           : (A.orb64[(size_t)pv * ORB64 + 12] != 0.0);
  R acc[NS];
#pragma unroll
  for (int s = 0; s < NS; ++s) acc[s] = R(0);
  int key = -1;
  for (int j = 0; j < LNL_PPT; ++j) {
    const int pt = blockIdx.x * LNL_CHUNK + j * LNL_THREADS + tid;
    const int lc = (valid && pt < A.npt) ? A.lcids[pt] : -1;
    const bool flush = key >= 0 && lc >= 0 && lc != key;
    if (__any_sync(0xffffffffu, flush)) {
      lnlike_flush<R, NS>(A, acc, key, flush, wred[warp]);
      if (flush) key = -1;
    }
    if (lc < 0) continue;
    lnlike_point<R, SPLIT, GRAD>(A, pv, pt, lc, lcs, lc_smem, orbc, dcs, acc);
    key = lc;
  }
  lnlike_flush<R, NS>(A, acc, key, key >= 0, wred[warp]);
  __syncthreads();
  double* out = A.partials + ((size_t)pv * gridDim.x + blockIdx.x) * (1 + A.ngrad);
  for (int i = tid; i <= A.ngrad; i += blockDim.x) {
    double sm = 0.0;
#pragma unroll
    for (int w = 0; w < LNL_NW; ++w) sm += wred[w][i];
    out[i] = sm;
  }
}

// Sum the block partials of each pv in a fixed order; invalid pv -> NaN.
__global__ void lnlike_reduce_kernel(const double* __restrict__ partials, int nblk, int ngrad, int npv,
                                     const double* __restrict__ cpart, int ncpart, const double* __restrict__ orb64,
                                     const float* __restrict__ orb32, double* __restrict__ lnl,
                                     double* __restrict__ grad) {
  const int pv = blockIdx.x;
  const bool valid = orb32 ? (__float_as_int(orb32[(size_t)pv * ORB32 + 14]) & FLAG_VALID)
                           : (orb64[(size_t)pv * ORB64 + 12] != 0.0);
  for (int i = threadIdx.x; i <= ngrad; i += blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nblk; ++b) s += partials[((size_t)pv * nblk + b) * (1 + ngrad) + i];
    if (!valid) s = CUDART_NAN;
    if (i == 0) {
      double c = 0.0;
      for (int b = 0; b < ncpart; ++b) c += cpart[b];
      lnl[pv] = s + c;
    }
    else if (grad) grad[(size_t)pv * ngrad + i - 1] = s;
  }
}

template <typename R>
struct GradWs {
  R *dc, *tab, *dis, *dobs, *isig2;
  double *partials, *cconst;   // cconst: the constant of lnL in per-block parts
};

template <typename R>
static GradWs<R> carve_grad(Carve& cv, int npv, int npb, int npar, int ng, int npt, int nblk, int ngrad) {
  GradWs<R> g;
  g.dc = cv.take<R>((size_t)npv * 50);
  g.tab = cv.take<R>((size_t)npv * npb * (1 + npar) * ng);
  g.dis = cv.take<R>((size_t)npv * npb * (npar > 0 ? npar : 1));
  g.dobs = cv.take<R>((size_t)npt);
  g.isig2 = cv.take<R>((size_t)npt);
  g.partials = cv.take<double>((size_t)npv * nblk * (1 + ngrad));
  g.cconst = cv.take<double>((size_t)(npt + OBS_CHUNK - 1) / OBS_CHUNK);
  return g;
}

}  // namespace rr

using namespace rr;

extern "C" {

int rr_lnlike_ngrad(int nkc, int nep, int npb, int npar) { return nkc + nep + 5 + npb * npar; }

size_t rr_lnlike_workspace_bytes(int split, int npv, int npb, int nlc, int nep, int ng, int npar, int npt,
                                 int nkc) {
  const int nblk = (npt + LNL_CHUNK - 1) / LNL_CHUNK;
  const int ngrad = rr_lnlike_ngrad(nkc, nep, npb, npar);
  size_t base = split ? rr_full_split_workspace_bytes(npv, npb, nlc, nep, ng) : rr_full_f64_workspace_bytes(npv, npb, ng);
  Carve c(nullptr);
  if (split) carve_grad<float>(c, npv, npb, npar, ng, npt, nblk, ngrad);
  else carve_grad<double>(c, npv, npb, npar, ng, npt, nblk, ngrad);
  return base + c.used + 512;
}

}  // extern "C"

template <typename R>
static int lnlike_impl(int split, int law, const double* ldc, int npar, const double* mu, const double* times,
                       const float* times_ff, double t_ref, double t_absmax, int npt, const double* k, int nkc,
                       const double* t0, int ldt0, int nep, const double* p, const double* a, const double* inc,
                       const double* e, const double* w, int npv, int nlc, int npb, const int32_t* lcids,
                       const int32_t* pbids, const int32_t* epids, const int32_t* nsamples,
                       const double* exptimes, const R* ldp, const R* istar, const R* weights, int nk, int ng,
                       int nz, double dk, double kmin, double kmax, double dg, const double* z_edges,
                       const double* obs, const double* sigma, void* workspace, size_t workspace_bytes,
                       double* lnl, double* grad, void* stream) {
  if (nkc > 1 && nkc != npb) return RR_ERR_SHAPE;
  if (law < 0 || law >= LD_NLAWS) return RR_ERR_LAW;
  if (npt < 1 || npv < 0 || nlc < 1 || npb < 1 || nk < 2 || ng < 2 || nz < 1 || nz > 64 || nkc < 1 || nep < 1 ||
      nep > ldt0 || npar < 0 || npar > MAX_GRAD_PAR)
    return RR_ERR_ARG;
  const int ngrad = rr_lnlike_ngrad(nkc, nep, npb, npar);
  if (ngrad > MAX_NGRAD) return RR_ERR_ARG;
  if (npv == 0) return RR_OK;
  if (npv > 65535) return RR_ERR_ARG;
  if (workspace_bytes < rr_lnlike_workspace_bytes(split, npv, npb, nlc, nep, ng, npar, npt, nkc))
    return RR_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  size_t base = split ? rr_full_split_workspace_bytes(npv, npb, nlc, nep, ng) : rr_full_f64_workspace_bytes(npv, npb, ng);
  int st;
  if (split)
    st = rr_prepare_split(t_ref, t_absmax, k, nkc, t0, ldt0, nep, p, a, inc, e, w, npv, nlc, npb, pbids, epids,
                          nsamples, exptimes, (const float*)ldp, (const float*)istar, (const float*)weights, nk, ng,
                          nz, dk, kmin, kmax, z_edges, workspace, base, stream, 0, nullptr, 0, nullptr, 0);
  else
    st = rr_prepare_f64(k, nkc, p, a, inc, e, w, npv, npb, (const double*)ldp, (const double*)weights, nk, ng, nz,
                        dk, kmin, kmax, z_edges, workspace, base, stream, 0, nullptr, 0, nullptr, 0);
  if (st) return st;
  const int nblk = (npt + LNL_CHUNK - 1) / LNL_CHUNK;
  Carve cv(static_cast<char*>(workspace) + base);
  GradWs<R> g = carve_grad<R>(cv, npv, npb, npar, ng, npt, nblk, ngrad);
  // prologue tables of the forward pass (inside the base workspace)
  Carve pcv(workspace);
  const double* orb64 = nullptr;
  const float *orb32 = nullptr, *lc32 = nullptr;
  const R* ldm;
  if (split) {
    orb32 = pcv.take<float>((size_t)npv * ORB32);
    lc32 = pcv.take<float>((size_t)npv * nlc * LC32);
    ldm = (const R*)pcv.take<float>((size_t)npv * npb * ng);
  } else {
    orb64 = pcv.take<double>((size_t)npv * ORB64);
    ldm = (const R*)pcv.take<double>((size_t)npv * npb * ng);
  }
  grad_orbit_kernel<R><<<(npv + 63) / 64, 64, 0, s>>>(p, a, inc, e, w, npv, g.dc);
  grad_ld_kernel<R><<<dim3(npv, npb), 128, 0, s>>>(law, ldc, npb, npar, mu, nz, ldp, k, nkc, weights, nk, ng, dk,
                                                   kmin, kmax, z_edges, g.tab, g.dis);
  const int nobs = (npt + OBS_CHUNK - 1) / OBS_CHUNK;
  obs_kernel<R><<<nobs, OBS_THREADS, 0, s>>>(obs, sigma, lcids, npt, g.dobs, g.isig2, g.cconst);
  GradArgs<R> A{};
  A.times = times; A.times_ff = reinterpret_cast<const float2*>(times_ff);
  A.lcids = lcids; A.pbids = pbids; A.epids = epids; A.nsamples = nsamples; A.exptimes = exptimes;
  A.dobs = g.dobs; A.isig2 = g.isig2;
  A.k = k; A.t0 = t0; A.p = p; A.istar64 = (const double*)istar; A.nkc = nkc; A.ldt0 = ldt0; A.nep = nep;
  A.orb64 = orb64; A.orb32 = orb32; A.lc32 = lc32;
  A.ldm = ldm; A.dc = g.dc; A.tab = g.tab; A.dis = g.dis;
  A.npt = npt; A.npv = npv; A.npb = npb; A.nlc = nlc; A.ng = ng; A.npar = npar; A.ngrad = ngrad;
  A.dg = dg; A.grad = grad != nullptr; A.partials = g.partials;
  dim3 grid(nblk, npv);
  if (split) {
    if (A.grad) lnlike_kernel<R, true, true><<<grid, LNL_THREADS, 0, s>>>(A);
    else lnlike_kernel<R, true, false><<<grid, LNL_THREADS, 0, s>>>(A);
  } else {
    if (A.grad) lnlike_kernel<R, false, true><<<grid, LNL_THREADS, 0, s>>>(A);
    else lnlike_kernel<R, false, false><<<grid, LNL_THREADS, 0, s>>>(A);
  }
  lnlike_reduce_kernel<<<npv, 64, 0, s>>>(g.partials, nblk, ngrad, npv, g.cconst, nobs, orb64, orb32, lnl, grad);
  return check_launch("rr_lnlike");
}

extern "C" {


int rr_lnlike_f64(int law, const double* ldc, int npar, const double* mu, const double* times, int npt,
                  const double* k, int nkc, const double* t0, int ldt0, int nep, const double* p, const double* a,
                  const double* inc, const double* e, const double* w, int npv, int nlc, int npb,
                  const int32_t* lcids, const int32_t* pbids, const int32_t* epids, const int32_t* nsamples,
                  const double* exptimes, const double* ldp, const double* istar, const double* weights, int nk,
                  int ng, int nz, double dk, double kmin, double kmax, double dg, const double* z_edges,
                  const double* obs, const double* sigma, void* workspace, size_t workspace_bytes, double* lnl,
                  double* grad, void* stream) {
  return lnlike_impl<double>(0, law, ldc, npar, mu, times, nullptr, 0.0, 0.0, npt, k, nkc, t0, ldt0, nep, p, a, inc,
                             e, w, npv, nlc, npb, lcids, pbids, epids, nsamples, exptimes, ldp, istar, weights, nk,
                             ng, nz, dk, kmin, kmax, dg, z_edges, obs, sigma, workspace, workspace_bytes, lnl, grad,
                             stream);
}

int rr_lnlike_split(int law, const double* ldc, int npar, const double* mu, const float* times_ff, double t_ref,
                    double t_absmax, int npt, const double* k, int nkc, const double* t0, int ldt0, int nep,
                    const double* p, const double* a, const double* inc, const double* e, const double* w, int npv,
                    int nlc, int npb, const int32_t* lcids, const int32_t* pbids, const int32_t* epids,
                    const int32_t* nsamples, const double* exptimes, const float* ldp, const float* istar,
                    const float* weights, int nk, int ng, int nz, double dk, double kmin, double kmax, double dg,
                    const double* z_edges, const double* obs, const double* sigma, void* workspace,
                    size_t workspace_bytes, double* lnl, double* grad, void* stream) {
  return lnlike_impl<float>(1, law, ldc, npar, mu, nullptr, times_ff, t_ref, t_absmax, npt, k, nkc, t0, ldt0, nep, p,
                            a, inc, e, w, npv, nlc, npb, lcids, pbids, epids, nsamples, exptimes, ldp, istar, weights,
                            nk, ng, nz, dk, kmin, kmax, dg, z_edges, obs, sigma, workspace, workspace_bytes, lnl,
                            grad, stream);
}

}  // extern "C"
