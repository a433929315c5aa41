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

// Per-pv prologue: kmean, max k, channel records, orbit and bounding box.
template <typename R>
__global__ void ts_prepare_kernel(const double* __restrict__ k, const double* __restrict__ t0,
                                  const double* __restrict__ p, const double* __restrict__ a,
                                  const double* __restrict__ inc, const double* __restrict__ e,
                                  const double* __restrict__ w, const R* __restrict__ istar, int npv, int npb,
                                  double exptime0, double t_ref, double t_absmax, R* __restrict__ orb,
                                  R* __restrict__ ch, double* __restrict__ kstat) {
  const int pv = blockIdx.x * blockDim.x + threadIdx.x;
  if (pv >= npv) return;
  const double* kp = k + (size_t)pv * npb;
  double km = 0.0, kx = kp[0];
  for (int b = 0; b < npb; ++b) { km += kp[b]; kx = fmax(kx, kp[b]); }
  km /= npb;
  kstat[pv] = km;
  kstat[npv + pv] = kx;
  for (int b = 0; b < npb; ++b) {
    R* c = ch + ((size_t)pv * npb + b) * TS_CH;
    c[0] = (R)(kp[b] * kp[b] / (km * km));
    c[1] = (R)(kp[b] - km);
    const R is = istar[(size_t)pv * npb + b];
    c[2] = isfinite((double)is) ? R(1) / is : R(CUDART_NAN);
    c[3] = R(0);
  }
  const bool valid = !(isnan(a[pv]) || a[pv] <= 1.0 || e[pv] < 0.0);
  R* o = orb + (size_t)pv * TS_ORB;
  for (int i = 0; i < TS_ORB; ++i) o[i] = R(0);
  o[15] = valid ? R(1) : R(0);
  if (!valid) return;
  double c[10];
  solve2d_conj(p[pv], a[pv], inc[pv], e[pv], w[pv], c);
  const double pad = 0.0015 + exptime0;
  const double t1 = contact_point(km, 1, c) - pad, t4 = contact_point(km, 4, c) + pad;
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

// One warp tile (128 points, 4 per lane) of one pv.  Out-of-box points get
// 1.0 in every channel (float4 stores per channel row); each in-box point is
// then evaluated by the whole warp: lane s computes sample s (z, area at
// kmean, its k-derivative, the table index), and lanes then take the channels,
// reading the samples back with shuffles.
template <typename R, bool SPLIT>
__global__ void __launch_bounds__(TS_WARPS * 32)
ts_flux_kernel(const double* __restrict__ times, const float2* __restrict__ times_ff, int npt,
               const double* __restrict__ t0, const double* __restrict__ p, int npv, int npb, int nsamples0,
               double exptime0, const R* __restrict__ orb_all, const R* __restrict__ ch_all,
               const R* __restrict__ ldm_all, int ng, double dg, R* __restrict__ flux, int ldflux) {
  const unsigned FULL = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pv = blockIdx.y + 65535 * blockIdx.z;
  if (pv >= npv) return;
  const R* o = orb_all + (size_t)pv * TS_ORB;
  const R* ch = ch_all + (size_t)pv * npb * TS_CH;
  const R* ldm = ldm_all + (size_t)pv * npb * ng;
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
  const bool vec_ok = ((ldflux & 3) == 0) && ((reinterpret_cast<uintptr_t>(flux) & 15) == 0) && sizeof(R) == 4;

  for (int tile = blockIdx.x * TS_WARPS + warp; tile < ntiles; tile += gridDim.x * TS_WARPS) {
    const int pt0 = tile * 128 + lane * 4;
    const bool full4 = pt0 + 4 <= npt;
    // ones (or NaN) for every channel
    const R fill = valid ? R(1) : R(CUDART_NAN);
    for (int b = 0; b < npb; ++b) {
      R* row = flux + ((size_t)pv * npb + b) * ldflux;
      if constexpr (sizeof(R) == 4) {
        if (full4 && vec_ok) {
          __stcs(reinterpret_cast<float4*>(row + pt0), make_float4(fill, fill, fill, fill));
          continue;
        }
      }
      for (int q = 0; q < 4; ++q)
        if (pt0 + q < npt) row[pt0 + q] = fill;
    }
    if (!valid) continue;
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
    // phase-folded times and in-box flags
    R tcq[4];
    unsigned inb = 0;
    for (int q = 0; q < 4; ++q) {
      tcq[q] = R(0);
      const int pt = pt0 + q;
      if (pt >= npt) continue;
      if (SPLIT) {
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
        tcq[q] = (R)t;
      } else {
        const double t = times[pt];
        const double tz = t0[pv], pp = p[pv];
        const double epoch = floor(__ddiv_rn(__dadd_rn(__dsub_rn(t, tz), __dmul_rn(0.5, pp)), pp));
        tcq[q] = (R)__dsub_rn(t, __dadd_rn(tz, __dmul_rn(epoch, pp)));
      }
      if (box_lo <= tcq[q] && tcq[q] <= box_hi) inb |= 1u << q;
    }
    __syncwarp();   // the ones above are visible before the in-box values overwrite them
    // in-box points, one at a time for the whole warp
    for (int q = 0; q < 4; ++q) {
      unsigned m = __ballot_sync(FULL, inb >> q & 1u);
      while (m) {
        const int src = __ffs(m) - 1;
        m &= m - 1;
        const R tc = __shfl_sync(FULL, tcq[q], src);
        const int pt = tile * 128 + src * 4 + q;
        for (int s0 = 0; s0 < nsamples0; s0 += 32) {
          const int ns_here = min(32, nsamples0 - s0);
          // lane s: sample s0 + s
          R ap0 = R(0), dadk = R(0), fr = R(0);
          int gi = 0, inner = 0;
          if (lane < ns_here) {
            const R t = tc + ex * ((R(s0 + lane) + R(0.5)) * inv_ns - R(0.5));
            R x = cc[4], y = cc[9];
            for (int mm = 3; mm >= 0; --mm) {
              x = x * t + cc[mm];
              y = y * t + cc[5 + mm];
            }
            const R z = sqrt(x * x + y * y);
            R kap;
            ap0 = ccia_star<R>(kmean, z, kap);
            dadk = R(2) * kmean * kap;
            if (z <= R(1) + kmean) {
              const R gg = z * inv1pk * inv_dg;
              gi = (int)gg;
              gi = min(max(gi, 0), ng - 2);
              fr = gg - (R)gi;
            } else {
              ap0 = R(0);
              dadk = R(0);
            }
            inner = (z <= inner_lim) ? 1 : 0;
          }
          for (int b0 = 0; b0 < npb; b0 += 32) {
            const int b = b0 + lane;
            R acc = R(0);
            const R* L = ldm + (size_t)(b < npb ? b : 0) * ng;
            const R* cr = ch + (size_t)(b < npb ? b : 0) * TS_CH;
            const R afac = cr[0], dkb = cr[1];
            for (int s = 0; s < ns_here; ++s) {
              const R a_s = __shfl_sync(FULL, ap0, s);
              const R d_s = __shfl_sync(FULL, dadk, s);
              const R f_s = __shfl_sync(FULL, fr, s);
              const int i_s = __shfl_sync(FULL, gi, s);
              const int in_s = __shfl_sync(FULL, inner, s);
              if (b < npb && a_s != R(0)) {
                const R l0 = L[i_s], l1 = L[i_s + 1];
                const R ip = l0 + f_s * (l1 - l0);
                const R area = in_s ? a_s * afac : a_s + dkb * d_s;
                acc += ip * area;
              }
            }
            if (b < npb) {
              R* dst = flux + ((size_t)pv * npb + b) * ldflux + pt;
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
  ts_prepare_kernel<R><<<(npv + 63) / 64, 64, 0, s>>>(k, t0, p, a, inc, e, w, istar, npv, npb, exptime0, t_ref,
                                                      t_absmax, orb, ch, kstat);
  // LD means at kmean: 3D table with the TS rule (kmin <= kmean <= max k), or the 2D table
  if constexpr (SPLIT)
    launch_ldm_f32(ldp, npv, npb, nz, kstat, 1, weights, nk, ng, dk, kmin, kmax, z_edges, weights ? 1 : 2,
                   kstat + npv, ldm, s);
  else
    launch_ldm_f64(ldp, npv, npb, nz, kstat, 1, weights, nk, ng, dk, kmin, kmax, z_edges, weights ? 1 : 2,
                   kstat + npv, ldm, s);
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
