// The full RoadRunner model (pytransit/models/roadrunner/model_full.py:9-100)
// on the GPU: per-parameter-vector prologue kernels (limb-darkening means,
// orbit + bounding box) and the per-point flux kernels, plain FP64 and split
// precision.
#include <cmath>

#include "rr_device.cuh"
#include "rr_internal.h"

namespace rr {

constexpr int LDM_PBB = 4;      // passbands per block of the LD-means kernel
constexpr int MAX_NZ = 64;      // radial grid points staged in shared memory

// ---------------------------------------------------------------------------
// Limb-darkening means, model_full.py:43-55:
//   ldm[pv, pb, :] = (1-ak) W[ik] @ ldp[pv, pb] + ak W[ik+1] @ ldp[pv, pb]
// with k = kw[pv * kw_stride], or a table built at k (calculate_weights_2d,
// common.py:153-185) when k is outside [kmin, kmax] (mode 0) or when ik+1
// would run past the table.  mode 1: the transmission-spectroscopy rule
// kmin <= k <= kmax_pv[pv] (model_trspec.py:48); mode 2: always the 2D table.
// Grid (npv, ceil(npb / LDM_PBB)), 128 threads.
// ---------------------------------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(128)
ldm_kernel(const R* __restrict__ ldp, int npb, int nz, const double* __restrict__ kw, int kw_stride,
           const R* __restrict__ W, int nk, int ng, double dk, double kmin, double kmax,
           const double* __restrict__ ze, int mode, const double* __restrict__ kmax_pv,
           R* __restrict__ ldm) {
  __shared__ R l[LDM_PBB][MAX_NZ];
  __shared__ double zes[MAX_NZ];
  const int pv = blockIdx.x;
  const int pb0 = blockIdx.y * LDM_PBB;
  const int nb = min(LDM_PBB, npb - pb0);
  for (int i = threadIdx.x; i < nb * nz; i += blockDim.x)
    l[i / nz][i % nz] = ldp[((size_t)pv * npb + pb0 + i / nz) * nz + i % nz];
  for (int i = threadIdx.x; i < nz; i += blockDim.x) zes[i] = ze[i];
  __syncthreads();

  const double k = kw[(size_t)pv * kw_stride];
  int ik = -1;
  double ak = 0.0;
  double kup = (mode == 1) ? kmax_pv[pv] : kmax;
  if (mode != 2 && W != nullptr && kmin <= k && k <= kup) {
    ik = (int)floor((k - kmin) / dk);
    ak = (k - kmin - ik * dk) / dk;
    if (ik + 1 >= nk || ik < 0) ik = -1;
  }
  R* out = ldm + ((size_t)pv * npb + pb0) * ng;
  if (ik >= 0) {
    const R* W0 = W + (size_t)ik * ng * nz;
    const R* W1 = W0 + (size_t)ng * nz;
    for (int j = threadIdx.x; j < nb * ng; j += blockDim.x) {
      int b = j / ng, g = j % ng;
      R d0 = R(0), d1 = R(0);
      const R* w0 = W0 + (size_t)g * nz;
      const R* w1 = W1 + (size_t)g * nz;
      for (int z = 0; z < nz; ++z) {
        d0 += __ldg(w0 + z) * l[b][z];
        d1 += __ldg(w1 + z) * l[b][z];
      }
      out[(size_t)b * ng + g] = (R(1) - (R)ak) * d0 + (R)ak * d1;
    }
  } else {
    // 2D table at this k, row by row in FP64: w_i = (A(ze_i) - A(ze_{i-1})) / sum
    const double gstep = (1.0 - 1e-7) / (double)(ng - 1);
    for (int g = threadIdx.x; g < ng; g += blockDim.x) {
      double gg = (g == ng - 1) ? (1.0 - 1e-7) : (double)g * gstep;
      double bb = gg * (1.0 + k);
      double acc[LDM_PBB] = {0.0, 0.0, 0.0, 0.0};
      double a0 = cci_acos(zes[0], k, bb);
      double s = a0;
      for (int b = 0; b < nb; ++b) acc[b] = a0 * (double)l[b][0];
      for (int z = 1; z < nz; ++z) {
        double a1 = cci_acos(zes[z], k, bb);
        double wz = a1 - a0;
        a0 = a1;
        s += wz;
        for (int b = 0; b < nb; ++b) acc[b] += wz * (double)l[b][z];
      }
      for (int b = 0; b < nb; ++b) out[(size_t)b * ng + g] = (R)(acc[b] / s);
    }
  }
}

// ---------------------------------------------------------------------------
// Orbit prologue, model_full.py:39-42 and 56-71, one thread per pv:
// validity, Taylor coefficients (solve2d), contact points (bounding_box).
// ---------------------------------------------------------------------------
struct OrbitArgs {
  const double *k, *t0, *p, *a, *inc, *e, *w, *exptimes;
  int nkc, ldt0, nep, npv, nlc, npb, nz;
  const void* ldp;       // validity probe ldp[pv, 0, 0] (double or float)
  int ldp_is_f32;
  // plain FP64 path
  double* orb64;
  // split path
  float *orb32, *box32, *ep32, *pb32;
  const float* istar32;
  double t_ref, t_absmax;
};

template <bool SPLIT>
__global__ void orbit_kernel(OrbitArgs A) {
  int pv = blockIdx.x * blockDim.x + threadIdx.x;
  if (pv >= A.npv) return;
  double a = A.a[pv], e = A.e[pv], p = A.p[pv];
  bool ldbad = A.ldp_is_f32 ? isnan(((const float*)A.ldp)[(size_t)pv * A.npb * A.nz])
                            : isnan(((const double*)A.ldp)[(size_t)pv * A.npb * A.nz]);
  bool valid = !(isnan(a) || a <= 1.0 || e < 0.0 || ldbad);
  double c[10];
  double t1 = 0.0, t4 = 0.0;
  double k0 = A.k[(size_t)pv * A.nkc];
  if (valid) {
    solve2d_conj(p, a, A.inc[pv], e, A.w[pv], c);
    t1 = contact_point(k0, 1, c);
    t4 = contact_point(k0, 4, c);
  } else {
    for (int i = 0; i < 10; ++i) c[i] = 0.0;
  }
  if (!SPLIT) {
    double* o = A.orb64 + (size_t)pv * ORB64;
    for (int i = 0; i < 10; ++i) o[i] = c[i];
    o[10] = t1;
    o[11] = t4;
    o[12] = valid ? 1.0 : 0.0;
    return;
  }
  float* o = A.orb32 + (size_t)pv * ORB32;
  for (int i = 0; i < 10; ++i) o[i] = (float)c[i];
  float p_hi = __double2float_rn(p);
  float p_lo = __double2float_rn(p - (double)p_hi);
  o[10] = p_hi;
  o[11] = p_lo;
  o[12] = __double2float_rn(1.0 / p);
  // epochs: d0 = t0 - t_ref as an FP32 pair
  double d0max = 0.0;
  for (int ep = 0; ep < A.nep; ++ep) {
    double d0 = A.t0[(size_t)pv * A.ldt0 + ep] - A.t_ref;
    float hi = __double2float_rn(d0);
    A.ep32[((size_t)pv * A.nep + ep) * 2 + 0] = hi;
    A.ep32[((size_t)pv * A.nep + ep) * 2 + 1] = __double2float_rn(d0 - (double)hi);
    d0max = fmax(d0max, fabs(d0));
  }
  // Bound of |fast-test tc - true tc|: 2^-24 (4 (T + |d0|) + 2 p), doubled.
  double err = ldexp(1.0, -21) * (A.t_absmax + d0max + p) + 1e-9;
  o[13] = (float)err;
  int flags = valid ? FLAG_VALID : 0;
  for (int lc = 0; lc < A.nlc; ++lc) {
    double pad = 0.003 + A.exptimes[lc];
    double lo = t1 - pad, hi = t4 + pad;
    A.box32[((size_t)pv * A.nlc + lc) * 2 + 0] = (float)lo;
    A.box32[((size_t)pv * A.nlc + lc) * 2 + 1] = (float)hi;
    if (hi + 2 * err >= 0.5 * p || lo - 2 * err <= -0.5 * p) flags |= FLAG_WIDE;
  }
  o[14] = __int_as_float(flags);
  o[15] = 0.0f;
  for (int pb = 0; pb < A.npb; ++pb) {
    double kk = A.k[(size_t)pv * A.nkc + (A.nkc == A.npb ? pb : 0)];
    float* q = A.pb32 + ((size_t)pv * A.npb + pb) * 4;
    q[0] = (float)kk;
    q[1] = (float)(1.0 / (1.0 + kk));
    // a non-finite disk integral makes every in-box point NaN, as (istar - I A)/istar does
    float is = A.istar32[(size_t)pv * A.npb + pb];
    q[2] = isfinite(is) ? 1.0f / is : __int_as_float(0x7fc00000);
    q[3] = 0.0f;
  }
}

// ---------------------------------------------------------------------------
// Plain FP64 flux, model_full.py:75-99, one thread per (pv, point).  The phase
// fold uses explicitly rounded operations so no multiply-add is fused: at
// BJD-scale times the reference's rounding sequence matters at 1e-10 d.
// ---------------------------------------------------------------------------
struct FluxF64Args {
  const double* times;
  const double *k, *t0, *p, *exptimes, *istar, *ldm, *orb64;
  const int32_t *lcids, *pbids, *epids, *nsamples;
  int npt, npv, nkc, ldt0, npb, ng, ldflux;
  double dg;
  double* flux;
};

// Parameter vector of a flux block: grid.y x grid.z cover npv beyond 65535.
__device__ __forceinline__ int block_pv() { return blockIdx.z * 65535 + blockIdx.y; }

__global__ void __launch_bounds__(256) flux_f64_kernel(FluxF64Args A) {
  const int pv = block_pv();
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
  const double is = A.istar[(size_t)pv * A.npb + pb];
  const double* lda = A.ldm + ((size_t)pv * A.npb + pb) * A.ng;
  const int ns = A.nsamples[lc];
  double c[10];
  for (int i = 0; i < 10; ++i) c[i] = o[i];
  double f = 0.0;
  for (int s = 1; s < ns + 1; ++s) {
    double toff = ex * ((s - 0.5) / ns - 0.5);
    double z = sep_c_f64(tc + toff, c);
    double ip = interp_ldm_f64(z / (1.0 + kk), A.dg, lda, A.ng);
    double kap;
    double ap = ccia_star<double>(kk, z, kap);
    f += (is - ip * ap) / is;
  }
  *out = f / ns;
}

// ---------------------------------------------------------------------------
// Split-precision flux.  A warp owns 128 consecutive points of one pv (4 per
// lane, float4 stores).  Per point: an FP32 fast test of the phase-folded time
// against the bounding box widened by a per-pv error bound; candidate points
// get the exact phase reduction in FP32 pairs (error-free transformations)
// and the exact box test; in-box points are compacted into a per-warp list
// and their (point, sample) pairs are spread over the 32 lanes, each lane
// evaluating one sample (z, table interpolation, area) in FP32; a segmented
// shuffle reduction sums the samples of each point.  Output F = 1 - deficit.
// ---------------------------------------------------------------------------
constexpr int SPLIT_WARPS = 8;
constexpr int SPLIT_PTS = 4;                 // points per lane
constexpr int WARP_TILE = 32 * SPLIT_PTS;    // points per warp

struct FluxSplitArgs {
  const float2* times_ff;
  const int32_t *lcids, *pbids, *epids, *nsamples;
  const double* exptimes;
  const float *orb32, *box32, *ep32, *pb32, *ldm;
  int npt, npv, npb, nlc, nep, ng, ldflux;
  float inv_dg;
  float* flux;
};

struct WarpList {
  float tc[WARP_TILE];
  int lc[WARP_TILE];
  int slot[WARP_TILE];
  int off[WARP_TILE + 1];
  float acc[WARP_TILE];
  float res[WARP_TILE];
};

__device__ __forceinline__ float lens_area_f32(float k, float z) {
  float kap;
  return ccia_star<float>(k, z, kap);
}

__global__ void __launch_bounds__(SPLIT_WARPS * 32) flux_split_kernel(FluxSplitArgs A) {
  __shared__ WarpList lists[SPLIT_WARPS];
  const unsigned FULL = 0xffffffffu;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int pv = block_pv();
  const int base = (blockIdx.x * SPLIT_WARPS + warp) * WARP_TILE;
  if (base >= A.npt || pv >= A.npv) return;  // warp-uniform
  const int pt0 = base + lane * SPLIT_PTS;
  const float* o = A.orb32 + (size_t)pv * ORB32;
  const int flags = __float_as_int(__ldg(o + 14));
  float* row = A.flux + (size_t)pv * A.ldflux;
  const bool vec = (pt0 + SPLIT_PTS <= A.npt) &&
                   ((reinterpret_cast<uintptr_t>(row + pt0) & 15) == 0);

  float res[SPLIT_PTS] = {1.0f, 1.0f, 1.0f, 1.0f};
  if (!(flags & FLAG_VALID)) {
    for (int q = 0; q < SPLIT_PTS; ++q) res[q] = __int_as_float(0x7fc00000);
  } else {
    const float p_hi = __ldg(o + 10), p_lo = __ldg(o + 11), inv_p = __ldg(o + 12), err = __ldg(o + 13);
    const bool wide = flags & FLAG_WIDE;
    float hi[SPLIT_PTS], lo[SPLIT_PTS];
    int lcv[SPLIT_PTS];
    if (pt0 + SPLIT_PTS <= A.npt && ((reinterpret_cast<uintptr_t>(A.times_ff + pt0) & 15) == 0) &&
        ((reinterpret_cast<uintptr_t>(A.lcids + pt0) & 15) == 0)) {
      float4 u = __ldg(reinterpret_cast<const float4*>(A.times_ff + pt0));
      float4 v = __ldg(reinterpret_cast<const float4*>(A.times_ff + pt0 + 2));
      int4 l4 = __ldg(reinterpret_cast<const int4*>(A.lcids + pt0));
      hi[0] = u.x; lo[0] = u.y; hi[1] = u.z; lo[1] = u.w;
      hi[2] = v.x; lo[2] = v.y; hi[3] = v.z; lo[3] = v.w;
      lcv[0] = l4.x; lcv[1] = l4.y; lcv[2] = l4.z; lcv[3] = l4.w;
    } else {
      for (int q = 0; q < SPLIT_PTS; ++q) {
        int pt = pt0 + q;
        if (pt < A.npt) {
          float2 tt = __ldg(A.times_ff + pt);
          hi[q] = tt.x; lo[q] = tt.y; lcv[q] = __ldg(A.lcids + pt);
        } else {
          hi[q] = 0.0f; lo[q] = 0.0f; lcv[q] = -1;
        }
      }
    }
    // fast test
    unsigned cand = 0;
    float nq[SPLIT_PTS];
#pragma unroll
    for (int q = 0; q < SPLIT_PTS; ++q) {
      nq[q] = 0.0f;
      if (lcv[q] < 0) continue;
      const int lc = lcv[q];
      const int ep = __ldg(A.epids + lc);
      const float d0h = __ldg(A.ep32 + ((size_t)pv * A.nep + ep) * 2);
      const float s = hi[q] - d0h;
      const float n = floorf(fmaf(s, inv_p, 0.5f));
      nq[q] = n;
      const float r = fmaf(-n, p_hi, s);
      const float2 bb = __ldg(reinterpret_cast<const float2*>(A.box32) + (size_t)pv * A.nlc + lc);
      if (wide || (r >= bb.x - err && r <= bb.y + err)) cand |= 1u << q;
    }
    if (__ballot_sync(FULL, cand != 0)) {
      WarpList& L = lists[warp];
      int nitems = 0;
      unsigned inbox = 0;
#pragma unroll
      for (int q = 0; q < SPLIT_PTS; ++q) {
        bool in = false;
        float tcv = 0.0f;
        if (cand >> q & 1u) {
          const int lc = lcv[q];
          const int ep = __ldg(A.epids + lc);
          const float d0h = __ldg(A.ep32 + ((size_t)pv * A.nep + ep) * 2);
          const float d0l = __ldg(A.ep32 + ((size_t)pv * A.nep + ep) * 2 + 1);
          float n = nq[q];
          // tc = (hi + lo) - (d0h + d0l) - n (p_hi + p_lo), FP32 pairs
          float s1, e1, q1, e2, s2, e3;
          two_sum(hi[q], -d0h, s1, e1);
          two_prod(n, p_hi, q1, e2);
          two_sum(s1, -q1, s2, e3);
          float tail = ((e1 + e3) - e2) + (lo[q] - d0l) - n * p_lo;
          float t = s2 + tail;
          // the fast epoch estimate can be off by one near phase +-1/2
          if (t >= 0.5f * p_hi) { n += 1.0f; }
          else if (t < -0.5f * p_hi) { n -= 1.0f; }
          if (n != nq[q]) {
            two_prod(n, p_hi, q1, e2);
            two_sum(s1, -q1, s2, e3);
            tail = ((e1 + e3) - e2) + (lo[q] - d0l) - n * p_lo;
            t = s2 + tail;
          }
          const float2 bb = __ldg(reinterpret_cast<const float2*>(A.box32) + (size_t)pv * A.nlc + lc);
          in = (bb.x <= t && t <= bb.y);
          tcv = t;
        }
        const unsigned m = __ballot_sync(FULL, in);
        if (in) {
          const int pos = nitems + __popc(m & ((1u << lane) - 1u));
          L.tc[pos] = tcv;
          L.lc[pos] = lcv[q];
          L.slot[pos] = lane * SPLIT_PTS + q;
          inbox |= 1u << q;
        }
        nitems += __popc(m);
      }
      __syncwarp();
      if (nitems > 0) {
        // exclusive prefix sum of the sample counts -> L.off
        int carry = 0;
        for (int c0 = 0; c0 < nitems; c0 += 32) {
          const int it = c0 + lane;
          const int v = (it < nitems) ? __ldg(A.nsamples + L.lc[it]) : 0;
          int incl = v;
#pragma unroll
          for (int d = 1; d < 32; d <<= 1) {
            int u = __shfl_up_sync(FULL, incl, d);
            if (lane >= d) incl += u;
          }
          if (it < nitems) {
            L.off[it] = carry + incl - v;
            L.acc[it] = 0.0f;
          }
          carry += __shfl_sync(FULL, incl, 31);
        }
        if (lane == 0) L.off[nitems] = carry;
        __syncwarp();
        const int total = carry;
        float c[10];
#pragma unroll
        for (int i = 0; i < 10; ++i) c[i] = __ldg(o + i);
        for (int f0 = 0; f0 < total; f0 += 32) {
          const int f = f0 + lane;
          float d = 0.0f;
          int item = -1;
          if (f < total) {
            // largest item with off[item] <= f
            int lo_i = 0, hi_i = nitems - 1;
            while (lo_i < hi_i) {
              int mid = (lo_i + hi_i + 1) >> 1;
              if (L.off[mid] <= f) lo_i = mid; else hi_i = mid - 1;
            }
            item = lo_i;
            const int s = f - L.off[item];
            const int lc = L.lc[item];
            const int ns = __ldg(A.nsamples + lc);
            const float ex = (float)__ldg(A.exptimes + lc);
            const int pb = __ldg(A.pbids + lc);
            const float4 pbr = __ldg(reinterpret_cast<const float4*>(A.pb32) + (size_t)pv * A.npb + pb);
            const float k = pbr.x, inv1pk = pbr.y;
            // time_offset = exptime ((isample - 0.5)/ns - 0.5), isample = s + 1
            const float t = L.tc[item] + ex * ((float(s) + 0.5f) / float(ns) - 0.5f);
            const float z = sep_c_f32(t, c);
            if (z < 1.0f + k) {
              const float gg = z * inv1pk * A.inv_dg;
              int i = (int)gg;
              i = min(max(i, 0), A.ng - 2);
              const float fr = gg - (float)i;
              const float* lda = A.ldm + ((size_t)pv * A.npb + pb) * A.ng;
              const float l0 = __ldg(lda + i), l1 = __ldg(lda + i + 1);
              const float ip = fmaf(fr, l1 - l0, l0);
              d = ip * lens_area_f32(k, z);
            }
          }
          // segmented sum over lanes holding the same item
#pragma unroll
          for (int dd = 1; dd < 32; dd <<= 1) {
            const float dv = __shfl_down_sync(FULL, d, dd);
            const int iv = __shfl_down_sync(FULL, item, dd);
            if (lane + dd < 32 && iv == item) d += dv;
          }
          const int iprev = __shfl_up_sync(FULL, item, 1);
          if (item >= 0 && (lane == 0 || iprev != item)) L.acc[item] += d;
          __syncwarp();
        }
        for (int it = lane; it < nitems; it += 32) {
          const int lc = L.lc[it];
          const int pb = __ldg(A.pbids + lc);
          const float inv_is = __ldg(A.pb32 + ((size_t)pv * A.npb + pb) * 4 + 2);
          const float ns = (float)__ldg(A.nsamples + lc);
          L.res[L.slot[it]] = 1.0f - L.acc[it] * inv_is / ns;
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < SPLIT_PTS; ++q)
          if (inbox >> q & 1u) res[q] = L.res[lane * SPLIT_PTS + q];
      }
      __syncwarp();
    }
  }
  if (vec) {
    __stcs(reinterpret_cast<float4*>(row + pt0), make_float4(res[0], res[1], res[2], res[3]));
  } else {
    for (int q = 0; q < SPLIT_PTS; ++q)
      if (pt0 + q < A.npt) __stcs(row + pt0 + q, res[q]);
  }
}

}  // namespace rr

using namespace rr;

extern "C" {

size_t rr_full_f64_workspace_bytes(int npv, int npb, int ng) {
  Carve c(nullptr);
  c.take<double>((size_t)npv * ORB64);
  c.take<double>((size_t)npv * npb * ng);
  return c.used + 256;
}

size_t rr_full_split_workspace_bytes(int npv, int npb, int nlc, int nep, int ng) {
  Carve c(nullptr);
  c.take<float>((size_t)npv * ORB32);
  c.take<float>((size_t)npv * nlc * 2);
  c.take<float>((size_t)npv * nep * 2);
  c.take<float>((size_t)npv * npb * 4);
  c.take<float>((size_t)npv * npb * ng);
  return c.used + 256;
}

static int check_common(int npt, int nkc, int npv, int nlc, int npb, int nk, int ng, int nz, int ldflux) {
  if (nkc > 1 && nkc != npb) return RR_ERR_SHAPE;
  if (npt < 0 || npv < 0 || nlc < 1 || npb < 1 || nk < 2 || ng < 2 || nz < 1 || nz > MAX_NZ ||
      nkc < 1 || ldflux < npt)
    return RR_ERR_ARG;
  return RR_OK;
}

struct SplitTables {
  float *orb, *box, *ep, *pb, *ldm;
};

static SplitTables carve_split(void* ws, int npv, int npb, int nlc, int nep, int ng) {
  Carve cv(ws);
  SplitTables t;
  t.orb = cv.take<float>((size_t)npv * ORB32);
  t.box = cv.take<float>((size_t)npv * nlc * 2);
  t.ep = cv.take<float>((size_t)npv * nep * 2);
  t.pb = cv.take<float>((size_t)npv * npb * 4);
  t.ldm = cv.take<float>((size_t)npv * npb * ng);
  return t;
}

int rr_prepare_f64(const double* k, int nkc, const double* p, const double* a, const double* inc,
                   const double* e, const double* w, int npv, int npb, const double* ldp,
                   const double* weights, int nk, int ng, int nz, double dk, double kmin, double kmax,
                   const double* z_edges, void* workspace, size_t workspace_bytes, void* stream) {
  if (nkc > 1 && nkc != npb) return RR_ERR_SHAPE;
  if (npv < 0 || npb < 1 || nk < 2 || ng < 2 || nz < 1 || nz > MAX_NZ || nkc < 1) return RR_ERR_ARG;
  if (npv == 0) return RR_OK;
  if (workspace_bytes < rr_full_f64_workspace_bytes(npv, npb, ng)) return RR_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  Carve cv(workspace);
  double* orb = cv.take<double>((size_t)npv * ORB64);
  double* ldm = cv.take<double>((size_t)npv * npb * ng);
  dim3 lg(npv, (npb + LDM_PBB - 1) / LDM_PBB);
  ldm_kernel<double><<<lg, 128, 0, s>>>(ldp, npb, nz, k, nkc, weights, nk, ng, dk, kmin, kmax, z_edges, 0,
                                        nullptr, ldm);
  OrbitArgs oa{};
  oa.k = k; oa.p = p; oa.a = a; oa.inc = inc; oa.e = e; oa.w = w;
  oa.nkc = nkc; oa.npv = npv; oa.npb = npb; oa.nz = nz;
  oa.ldp = ldp; oa.ldp_is_f32 = 0; oa.orb64 = orb;
  orbit_kernel<false><<<(npv + 31) / 32, 32, 0, s>>>(oa);
  return check_launch("rr_prepare_f64");
}

int rr_flux_f64(const double* times, int npt, const double* k, int nkc, const double* t0, int ldt0,
                const double* p, int npv, int nlc, int npb, const int32_t* lcids, const int32_t* pbids,
                const int32_t* epids, const int32_t* nsamples, const double* exptimes,
                const double* istar, int ng, double dg, const void* workspace, double* flux, int ldflux,
                void* stream) {
  if (nkc > 1 && nkc != npb) return RR_ERR_SHAPE;
  if (npt < 0 || npv < 0 || nlc < 1 || npb < 1 || ng < 2 || nkc < 1 || ldflux < npt) return RR_ERR_ARG;
  if (npv == 0 || npt == 0) return RR_OK;
  Carve cv(const_cast<void*>(workspace));
  double* orb = cv.take<double>((size_t)npv * ORB64);
  double* ldm = cv.take<double>((size_t)npv * npb * ng);
  FluxF64Args fa{};
  fa.times = times; fa.k = k; fa.t0 = t0; fa.p = p; fa.exptimes = exptimes; fa.istar = istar;
  fa.ldm = ldm; fa.orb64 = orb; fa.lcids = lcids; fa.pbids = pbids; fa.epids = epids;
  fa.nsamples = nsamples; fa.npt = npt; fa.npv = npv; fa.nkc = nkc; fa.ldt0 = ldt0; fa.npb = npb;
  fa.ng = ng; fa.ldflux = ldflux; fa.dg = dg; fa.flux = flux;
  dim3 fg((npt + 255) / 256, npv < 65535 ? npv : 65535, (npv + 65534) / 65535);
  flux_f64_kernel<<<fg, 256, 0, as_stream(stream)>>>(fa);
  return check_launch("rr_flux_f64");
}

int rr_full_f64(const double* times, int npt, const double* k, int nkc, const double* t0, int ldt0,
                const double* p, const double* a, const double* inc, const double* e, const double* w,
                int npv, int nlc, int npb, const int32_t* lcids, const int32_t* pbids,
                const int32_t* epids, const int32_t* nsamples, const double* exptimes,
                const double* ldp, const double* istar, const double* weights, int nk, int ng, int nz,
                double dk, double kmin, double kmax, double dg, const double* z_edges, void* workspace,
                size_t workspace_bytes, double* flux, int ldflux, void* stream) {
  int st = check_common(npt, nkc, npv, nlc, npb, nk, ng, nz, ldflux);
  if (st) return st;
  if (npv == 0 || npt == 0) return RR_OK;
  if (workspace_bytes < rr_full_f64_workspace_bytes(npv, npb, ng)) return RR_ERR_WORKSPACE;
  st = rr_prepare_f64(k, nkc, p, a, inc, e, w, npv, npb, ldp, weights, nk, ng, nz, dk, kmin, kmax, z_edges,
                      workspace, workspace_bytes, stream);
  if (st) return st;
  return rr_flux_f64(times, npt, k, nkc, t0, ldt0, p, npv, nlc, npb, lcids, pbids, epids, nsamples, exptimes,
                     istar, ng, dg, workspace, flux, ldflux, stream);
}

int rr_prepare_split(double t_ref, double t_absmax, const double* k, int nkc, const double* t0, int ldt0,
                     int nep, const double* p, const double* a, const double* inc, const double* e,
                     const double* w, int npv, int nlc, int npb, const double* exptimes, const float* ldp,
                     const float* istar, const float* weights, int nk, int ng, int nz, double dk,
                     double kmin, double kmax, const double* z_edges, void* workspace,
                     size_t workspace_bytes, void* stream) {
  if (nkc > 1 && nkc != npb) return RR_ERR_SHAPE;
  if (npv < 0 || nlc < 1 || npb < 1 || nk < 2 || ng < 2 || nz < 1 || nz > MAX_NZ || nkc < 1 || nep < 1 ||
      nep > ldt0)
    return RR_ERR_ARG;
  if (npv == 0) return RR_OK;
  if (workspace_bytes < rr_full_split_workspace_bytes(npv, npb, nlc, nep, ng)) return RR_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  SplitTables t = carve_split(workspace, npv, npb, nlc, nep, ng);
  dim3 lg(npv, (npb + LDM_PBB - 1) / LDM_PBB);
  ldm_kernel<float><<<lg, 128, 0, s>>>(ldp, npb, nz, k, nkc, weights, nk, ng, dk, kmin, kmax, z_edges, 0,
                                       nullptr, t.ldm);
  OrbitArgs oa{};
  oa.k = k; oa.t0 = t0; oa.p = p; oa.a = a; oa.inc = inc; oa.e = e; oa.w = w; oa.exptimes = exptimes;
  oa.nkc = nkc; oa.ldt0 = ldt0; oa.nep = nep; oa.npv = npv; oa.nlc = nlc; oa.npb = npb; oa.nz = nz;
  oa.ldp = ldp; oa.ldp_is_f32 = 1; oa.orb32 = t.orb; oa.box32 = t.box; oa.ep32 = t.ep; oa.pb32 = t.pb;
  oa.istar32 = istar; oa.t_ref = t_ref; oa.t_absmax = t_absmax;
  orbit_kernel<true><<<(npv + 31) / 32, 32, 0, s>>>(oa);
  return check_launch("rr_prepare_split");
}

int rr_flux_split(const float* times_ff, int npt, const int32_t* lcids, const int32_t* pbids,
                  const int32_t* epids, const int32_t* nsamples, const double* exptimes, int npv, int nlc,
                  int npb, int nep, int ng, double dg, const void* workspace, float* flux, int ldflux,
                  void* stream) {
  if (npt < 0 || npv < 0 || nlc < 1 || npb < 1 || ng < 2 || nep < 1 || ldflux < npt) return RR_ERR_ARG;
  if (npv == 0 || npt == 0) return RR_OK;
  SplitTables t = carve_split(const_cast<void*>(workspace), npv, npb, nlc, nep, ng);
  FluxSplitArgs fa{};
  fa.times_ff = reinterpret_cast<const float2*>(times_ff);
  fa.lcids = lcids; fa.pbids = pbids; fa.epids = epids; fa.nsamples = nsamples; fa.exptimes = exptimes;
  fa.orb32 = t.orb; fa.box32 = t.box; fa.ep32 = t.ep; fa.pb32 = t.pb; fa.ldm = t.ldm;
  fa.npt = npt; fa.npv = npv; fa.npb = npb; fa.nlc = nlc; fa.nep = nep; fa.ng = ng; fa.ldflux = ldflux;
  fa.inv_dg = (float)(1.0 / dg); fa.flux = flux;
  dim3 fg((npt + WARP_TILE * SPLIT_WARPS - 1) / (WARP_TILE * SPLIT_WARPS), npv < 65535 ? npv : 65535,
          (npv + 65534) / 65535);
  flux_split_kernel<<<fg, SPLIT_WARPS * 32, 0, as_stream(stream)>>>(fa);
  return check_launch("rr_flux_split");
}

int rr_full_split(const float* times_ff, double t_ref, double t_absmax, int npt, const double* k, int nkc,
                  const double* t0, int ldt0, int nep, const double* p, const double* a, const double* inc,
                  const double* e, const double* w, int npv, int nlc, int npb, const int32_t* lcids,
                  const int32_t* pbids, const int32_t* epids, const int32_t* nsamples,
                  const double* exptimes, const float* ldp, const float* istar, const float* weights,
                  int nk, int ng, int nz, double dk, double kmin, double kmax, double dg,
                  const double* z_edges, void* workspace, size_t workspace_bytes, float* flux,
                  int ldflux, void* stream) {
  int st = check_common(npt, nkc, npv, nlc, npb, nk, ng, nz, ldflux);
  if (st) return st;
  if (nep < 1 || nep > ldt0) return RR_ERR_ARG;
  if (npv == 0 || npt == 0) return RR_OK;
  if (workspace_bytes < rr_full_split_workspace_bytes(npv, npb, nlc, nep, ng)) return RR_ERR_WORKSPACE;
  st = rr_prepare_split(t_ref, t_absmax, k, nkc, t0, ldt0, nep, p, a, inc, e, w, npv, nlc, npb, exptimes, ldp,
                        istar, weights, nk, ng, nz, dk, kmin, kmax, z_edges, workspace, workspace_bytes,
                        stream);
  if (st) return st;
  return rr_flux_split(times_ff, npt, lcids, pbids, epids, nsamples, exptimes, npv, nlc, npb, nep, ng, dg,
                       workspace, flux, ldflux, stream);
}

}  // extern "C"
