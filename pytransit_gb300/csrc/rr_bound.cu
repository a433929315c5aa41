// Stated flux-error bounds of the split-precision paths: for every parameter
// vector, an upper bound of |F_split - F_FP64| over all its points, where
// F_FP64 is the plain FP64 path (which follows the reference's FP64
// arithmetic, model_full.py:75-99 and model_trspec.py:72-93, to ~1e-15).
//
// The bound is built from the split path's own prologue tables and the FP64
// parameters (the FP64 jet a lane per parameter vector, the rest a warp per
// parameter vector):
//   * the z error: the FP32 Taylor coefficients against the FP64 jet
//     recomputed here (the difference itself, not an estimate of it) summed
//     over the bounding box, |t|^j sum_j |dc_j|, plus the FP32 Horner, the
//     FP32 sample time and the square root: dz <= sum_j |dc_j| tb^j
//     + 4u M + u tb V + 4u (1 + k) + 1e-11 V, with u = 2^-24,
//     M = sum_j |c_j| tb^j and V = sum_j j |c_j| tb^(j-1) (the largest sky
//     speed), tb the largest |t| a sample of the box reaches;
//   * the flux's sensitivity to z on every LD-table row j (a sample in row j
//     has z in [z_j, z_j+1]): |dF/dz| <= (2 min(k, 1) I + A |dI/dz|) / istar
//     with I <= max(L_j, L_j+1), A <= A(z_j) (the area falls with z) and
//     |dI/dz| = |L_j+1 - L_j| / (dg (1 + k));
//   * the deficit's FP32 relative error: (64 + ns) u I A / istar per row (the
//     FP32 tables, lerp, kite area, disk integral and the sum over the ns
//     samples);
//   * the lerp position's rounding: 3u (g / dg) |L_j+1 - L_j| A / istar;
//   * the FP32 result's own rounding, u.
// The transmission-spectroscopy bound takes per channel the first-order area
// A_b <= max(afac A, A + |k_b - kmean| 2 pi kmean) and adds the k-derivative
// term's change near contact, |k_b - kmean| 2 kmean dkappa I / istar, with
// dkappa <= sqrt(2 dz / (kmean (1 - kmean))) (kappa_0 has a square-root
// singularity at the contacts, so this term, not the area, sets the TS bound).
#include <cmath>

#include "rr_device.cuh"
#include "rr_internal.h"
#include "rr_ts.cuh"

namespace rr {

constexpr double BOUND_U = 5.9604644775390625e-8;   // 2^-24

struct BoundArgs {
  const double *p, *a, *inc, *e, *w;
  const float *orb, *lc, *ldm;   // split RR: orb32 [npv][ORB32], lc32 [npv][nlc][LC32]; TS: orb [npv][TS_ORB], ch [npv][npb][TS_CH]
  int npv, npb, nlc, ng, ts, nsamples0;
  double dg, exptime0;
  double* bound;                 // [npv]
  unsigned long long* bound_max; // max over pv (bits of a non-negative double), zeroed by the caller
};

// The z error of pv on |t| <= tb, without the square root's term
// 4u (1 + kmax), which the per-pv pass adds: the FP32 coefficients of the
// record against the FP64 jet.
__device__ inline double z_error_part(const BoundArgs& B, int pv, const float* c32, double tb) {
  double c[10];
  solve2d_conj(B.p[pv], B.a[pv], B.inc[pv], B.e[pv], B.w[pv], c);
  double dcz = 0.0, M = 0.0, V = 0.0, tp = 1.0;
  for (int j = 0; j < 5; ++j) {
    dcz += (fabs((double)c32[j] - c[j]) + fabs((double)c32[5 + j] - c[5 + j])) * tp;
    M += (fabs(c[j]) + fabs(c[5 + j])) * tp;
    if (j < 4) V += (j + 1) * (fabs(c[j + 1]) + fabs(c[6 + j])) * tp;
    tp *= tb;
  }
  return dcz + 4 * BOUND_U * M + BOUND_U * tb * V + 1e-11 * V;
}

// Per-row terms in FP32 (the FP64 rate of this GPU is 1/64 of its FP32
// rate): every term is a sum of products of non-negative values, so its FP32
// value is within 16 ulps of the exact one and the result is raised by
// BOUND_SAFETY.  The z error dz is computed in FP64 and rounded up.
constexpr float BOUND_SAFETY = 1.0f + 1e-4f;

// A block takes one parameter vector per warp (at most 32).  First the FP64
// part of each z error, one lane of warp 0 per pv, so that every FP64
// instruction serves up to 32 pvs (the FP64 pipe is the scarce one); then a
// warp per pv over the LD-table rows.  RoadRunner populations take 32 pvs a
// block; transmission-spectroscopy ones, with every channel on every row,
// take 4, which spreads few pvs over more SMs.
constexpr int BOUND_PV_MAX = 32;

__global__ void __launch_bounds__(BOUND_PV_MAX * 32) error_bound_kernel(BoundArgs B) {
  __shared__ double s_dz[BOUND_PV_MAX];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int npb_blk = blockDim.x >> 5;   // pvs of this block
  const int pv0 = blockIdx.x * npb_blk;
  const unsigned FULL = 0xffffffffu;
  if (warp == 0) {
    const int pv = pv0 + lane;
    double part = 0.0;
    if (lane < npb_blk && pv < B.npv) {
      if (!B.ts) {
        const float* o = B.orb + (size_t)pv * ORB32;
        if (__float_as_int(o[14]) & FLAG_VALID) {
          const float* L0 = B.lc + (size_t)pv * B.nlc * LC32;
          double tb = 0.0;
          for (int lc = 0; lc < B.nlc; ++lc) {
            const float* r = L0 + (size_t)lc * LC32;
            tb = fmax(tb, fmax(fabs((double)r[LC_LO]), fabs((double)r[LC_HI])) + 0.5 * r[LC_EXPT]);
          }
          part = z_error_part(B, pv, o, tb);
        }
      } else {
        const float* o = B.orb + (size_t)pv * TS_ORB;
        if (o[15] != 0.0f) {
          const double tb = fmax(fabs((double)o[10]), fabs((double)o[11])) + 0.5 * B.exptime0;
          part = z_error_part(B, pv, o, tb);
        }
      }
    }
    if (lane < npb_blk) s_dz[lane] = part;
  }
  __syncthreads();
  const float u = (float)BOUND_U;
  const int ng = B.ng;
  const float dg = (float)B.dg;
  {
    const int i = warp;
    const int pv = pv0 + i;
    if (pv >= B.npv) return;   // warp-uniform
    float worst = 0.0f;
    if (!B.ts) {
      const float* o = B.orb + (size_t)pv * ORB32;
      const bool valid = __float_as_int(o[14]) & FLAG_VALID;
      if (valid) {
        const float* L0 = B.lc + (size_t)pv * B.nlc * LC32;
        double kmax = 0.0;
        for (int lc = 0; lc < B.nlc; ++lc) kmax = fmax(kmax, (double)L0[(size_t)lc * LC32 + LC_K]);
        const float dz = __double2float_ru(s_dz[i] + 4 * BOUND_U * (1.0 + kmax));
        for (int lc = 0; lc < B.nlc; ++lc) {
          const float* r = L0 + (size_t)lc * LC32;
          const float k = r[LC_K], inv_is = fabsf(r[LC_INVIS]);
          if (!isfinite(inv_is)) continue;   // every in-box value is NaN on both paths
          const int ns = __float_as_int(r[LC_NS]), pb = __float_as_int(r[LC_PB]);
          const float* L = B.ldm + ((size_t)pv * B.npb + pb) * ng;
          const float gz = dg * (1.0f + k), inv_gz = 1.0f / gz, k2 = 2.0f * fminf(k, 1.0f);
          const float cr = (64 + ns) * u;
          for (int j = lane; j < ng - 1; j += 32) {
            const float l0 = L[j], l1 = L[j + 1];
            const float Lm = fmaxf(fabsf(l0), fabsf(l1)), dL = fabsf(l1 - l0);
            float kap;
            const float ai = ccia_star<float>(k, (float)j * gz, kap) * inv_is;
            const float S = k2 * Lm * inv_is + ai * dL * inv_gz;
            const float e = cr * Lm * ai + S * dz + 3.0f * u * (float)(j + 1) * dL * ai;
            worst = fmaxf(worst, e);
          }
        }
      }
    } else {
      const float* o = B.orb + (size_t)pv * TS_ORB;
      const bool valid = o[15] != 0.0f;
      if (valid) {
        const float km = o[12];
        const float* ch = B.lc + (size_t)pv * B.npb * TS_CH;
        float afmax = 1.0f;
        for (int b = lane; b < B.npb; b += 32) afmax = fmaxf(afmax, ch[b * TS_CH]);
        for (int off = 16; off > 0; off >>= 1) afmax = fmaxf(afmax, __shfl_xor_sync(FULL, afmax, off));
        const double kmax = (double)km * sqrt((double)afmax);
        const double dz64 = s_dz[i] + 4 * BOUND_U * (1.0 + kmax);
        const float dz = __double2float_ru(dz64);
        // kappa_0 near the outer (inner) contact goes as sqrt(2 eps / (k (1 +- k))):
        // a z error dz moves it by at most sqrt(2 dz / (k (1 - k)))
        const float dkap = __double2float_ru(sqrt(2.0 * dz64 / ((double)km * fmax(1.0 - (double)km, 1e-3))));
        const float cr = (64 + B.nsamples0) * u;
        const float gz = dg * (1.0f + km), inv_gz = 1.0f / gz;
        const float ring = 2.0f * float(PI) * km;
        // lanes over the table rows, the channels inner: the area at the row's
        // z is shared by every channel
        for (int j = lane; j < ng - 1; j += 32) {
          float kap;
          const float A0 = ccia_star<float>(km, (float)j * gz, kap);
          const float rj = 3.0f * u * (float)(j + 1);
          const float* L = B.ldm + (size_t)pv * B.npb * ng + j;
          for (int b = 0; b < B.npb; ++b, L += ng) {
            const float afac = ch[b * TS_CH], dk = fabsf(ch[b * TS_CH + 1]), inv_is = fabsf(ch[b * TS_CH + 2]);
            if (!isfinite(inv_is)) continue;
            const float kb = km * sqrtf(afac);
            const float l0 = L[0], l1 = L[1];
            const float Lm = fmaxf(fabsf(l0), fabsf(l1)), dL = fabsf(l1 - l0);
            const float ai = fmaxf(afac * A0, fmaf(dk, ring, A0)) * inv_is;
            const float S = 2.0f * fminf(fmaxf(kb, km), 1.0f) * Lm * inv_is + ai * dL * inv_gz;
            const float e = cr * Lm * ai + S * dz + rj * dL * ai + dk * 2.0f * km * dkap * Lm * inv_is;
            worst = fmaxf(worst, e);
          }
        }
      }
    }
    for (int off = 16; off > 0; off >>= 1) worst = fmaxf(worst, __shfl_xor_sync(FULL, worst, off));
    if (lane == 0) {
      const double bnd = worst > 0.0f ? (double)(worst * BOUND_SAFETY) + BOUND_U : 0.0;
      B.bound[pv] = bnd;
      if (B.bound_max) atomicMax(B.bound_max, (unsigned long long)__double_as_longlong(bnd));
    }
  }
}

static int launch_bounds(BoundArgs& B, void* stream) {
  if (B.npv < 0 || B.npb < 1 || B.ng < 2 || !B.bound || !B.p || !B.a || !B.inc || !B.e || !B.w) return RR_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (B.bound_max) {
    const cudaError_t e = cudaMemsetAsync(B.bound_max, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) {
      set_cuda_error(e, "rr_error_bounds");
      return RR_ERR_CUDA;
    }
  }
  if (B.npv == 0) return RR_OK;
  const int per = B.ts ? 4 : BOUND_PV_MAX;
  const unsigned nblk = (unsigned)((B.npv + per - 1) / per);
  error_bound_kernel<<<nblk, per * 32, 0, s>>>(B);
  return check_launch("rr_error_bounds");
}

}  // namespace rr

using namespace rr;

extern "C" {

int rr_split_error_bounds(const double* p, const double* a, const double* inc, const double* e, const double* w,
                          int npv, int npb, int nlc, int nep, int ng, double dg, const void* workspace,
                          double* bound, double* bound_max, void* stream) {
  (void)nep;
  if (nlc < 1) return RR_ERR_ARG;
  BoundArgs B{};
  B.p = p; B.a = a; B.inc = inc; B.e = e; B.w = w;
  const float *orb = nullptr, *lc = nullptr, *ldm = nullptr;
  rr_full_split_tables(const_cast<void*>(workspace), npv, npb, nlc, nep, ng, &orb, &lc, &ldm);
  B.orb = orb; B.lc = lc; B.ldm = ldm;
  B.npv = npv; B.npb = npb; B.nlc = nlc; B.ng = ng; B.ts = 0; B.dg = dg;
  B.bound = bound;
  B.bound_max = reinterpret_cast<unsigned long long*>(bound_max);
  return launch_bounds(B, stream);
}

int rr_ts_split_error_bounds(const double* p, const double* a, const double* inc, const double* e, const double* w,
                             int npv, int npb, int ng, double dg, int nsamples0, double exptime0,
                             const void* workspace, double* bound, double* bound_max, void* stream) {
  if (nsamples0 < 1) return RR_ERR_ARG;
  BoundArgs B{};
  B.p = p; B.a = a; B.inc = inc; B.e = e; B.w = w;
  const void *orb = nullptr, *ch = nullptr, *ldm = nullptr;
  rr_ts_tables(const_cast<void*>(workspace), 1, npv, npb, ng, &orb, &ch, &ldm);
  B.orb = static_cast<const float*>(orb); B.lc = static_cast<const float*>(ch);
  B.ldm = static_cast<const float*>(ldm);
  B.npv = npv; B.npb = npb; B.nlc = 1; B.ng = ng; B.ts = 1; B.dg = dg;
  B.nsamples0 = nsamples0; B.exptime0 = exptime0;
  B.bound = bound;
  B.bound_max = reinterpret_cast<unsigned long long*>(bound_max);
  return launch_bounds(B, stream);
}

}  // extern "C"
