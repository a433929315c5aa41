// The full RoadRunner model (pytransit/models/roadrunner/model_full.py:9-100)
// on the GPU: per-parameter-vector prologue kernels (limb-darkening means,
// orbit + bounding box) and the per-point flux kernels, plain FP64 and split
// precision.
#include <algorithm>
#include <cmath>

#include "rr_device.cuh"
#include "rr_internal.h"
#include "rr_ts.cuh"

namespace rr {

constexpr int LDM_PBB = 4;      // passbands per block of the LD-means kernel
constexpr int MAX_NZ = 64;      // radial grid points staged in shared memory
constexpr int LDM_SCRATCH = 2048;   // FP64 areas of the 2D table per chunk of rows (FP32 tables)

// ---------------------------------------------------------------------------
// Limb-darkening means, model_full.py:43-55:
//   ldm[pv, pb, :] = (1-ak) W[ik] @ ldp[pv, pb] + ak W[ik+1] @ ldp[pv, pb]
// with k = kw[pv * kw_stride], or a table built at k (calculate_weights_2d,
// common.py:153-185) when k is outside [kmin, kmax] (mode 0) or when ik+1
// would run past the table.  mode 1: the transmission-spectroscopy rule
// kmin <= k <= kmax_pv[pv] (model_trspec.py:48); mode 2: always the 2D table.
// One block per (pv, share of the passband groups): the k-interpolated weight
// slab (or the 2D table, computed once per block) is staged in shared memory
// with coalesced loads (rows padded to nz+1 words so the dot products are
// free of bank conflicts), then the block walks its groups of LDM_PBB
// passbands and every (pb, g) output is a dot product from shared memory:
// ldm[pv][pb][g].
// ---------------------------------------------------------------------------
// Byte offset of the FP64 scratch after the slab [ng][nz+1] and the LD
// profiles [LDM_PBB][MAX_NZ] (8-byte aligned).
template <typename R>
__host__ __device__ inline size_t ldm_scratch_offset(int ng, int nz) {
  return (sizeof(R) * ((size_t)ng * (nz + 1) + (size_t)LDM_PBB * MAX_NZ) + 7) & ~size_t(7);
}

template <typename R>
__global__ void __launch_bounds__(128)
ldm_kernel(const R* __restrict__ ldp, int npb, int nz, const double* __restrict__ kw, int kw_stride,
           const R* __restrict__ W, int nk, int ng, double dk, double kmin, double kmax,
           const double* __restrict__ ze, int mode, const double* __restrict__ kmax_pv,
           R* __restrict__ ldm) {
  extern __shared__ __align__(16) unsigned char ldm_smem[];
  R* Wk = reinterpret_cast<R*>(ldm_smem);                  // [ng][nz + 1]
  R* l = Wk + (size_t)ng * (nz + 1);                       // [LDM_PBB][nz]
  const int ldw = nz + 1;
  const int pv = blockIdx.x;

  const double k = kw[(size_t)pv * kw_stride];
  int ik = -1;
  double ak = 0.0;
  double kup = (mode == 1) ? kmax_pv[pv] : kmax;
  if (mode != 2 && W != nullptr && kmin <= k && k <= kup) {
    ik = (int)floor((k - kmin) / dk);
    ak = (k - kmin - ik * dk) / dk;
    if (ik + 1 >= nk || ik < 0) ik = -1;
  }
  if (ik >= 0) {
    const R* W0 = W + (size_t)ik * ng * nz;
    const R* W1 = W0 + (size_t)ng * nz;
    const R a1 = (R)ak, a0 = R(1) - (R)ak;
    for (int i = threadIdx.x; i < ng * nz; i += blockDim.x)
      Wk[(i / nz) * ldw + (i % nz)] = a0 * __ldg(W0 + i) + a1 * __ldg(W1 + i);
  } else {
    // 2D table at this k (calculate_weights_2d, common.py:153-185) in FP64:
    // the areas A(ze_z) at every (g, z) in parallel, then per row the
    // differences w_z = A(ze_z) - A(ze_{z-1}) and their sum, normalised.  The
    // areas go to the table itself (FP64) or, for an FP32 table, to an FP64
    // scratch in chunks of rows.
    const double gstep = (1.0 - 1e-7) / (double)(ng - 1);
    double* A2 = (sizeof(R) == 8) ? reinterpret_cast<double*>(Wk)
                                  : reinterpret_cast<double*>(ldm_smem + ldm_scratch_offset<R>(ng, nz));
    const int rows = (sizeof(R) == 8) ? ng : max(1, LDM_SCRATCH / nz);
    const int lda = (sizeof(R) == 8) ? ldw : nz;
    for (int g0 = 0; g0 < ng; g0 += rows) {
      const int nr = min(rows, ng - g0);
      for (int i = threadIdx.x; i < nr * nz; i += blockDim.x) {
        const int g = g0 + i / nz, z = i % nz;
        const double gg = (g == ng - 1) ? 1.0 - 1e-7 : (double)g * gstep;
        A2[(size_t)(i / nz) * lda + z] = cci_acos(ze[z], k, gg * (1.0 + k));
      }
      __syncthreads();
      for (int rr = threadIdx.x; rr < nr; rr += blockDim.x) {
        const double* a = A2 + (size_t)rr * lda;
        R* row = Wk + (size_t)(g0 + rr) * ldw;
        double s = a[0];
        for (int z = 1; z < nz; ++z) s += a[z] - a[z - 1];
        // in place for an FP64 table: walk down so a[z-1] is still the area
        for (int z = nz - 1; z >= 1; --z) row[z] = (R)((a[z] - a[z - 1]) / s);
        row[0] = (R)(a[0] / s);
      }
      __syncthreads();
    }
  }
  const int ngroups = (npb + LDM_PBB - 1) / LDM_PBB;
  for (int grp = blockIdx.y; grp < ngroups; grp += gridDim.y) {
    const int pb0 = grp * LDM_PBB;
    const int nb = min(LDM_PBB, npb - pb0);
    __syncthreads();   // the slab is complete; the previous group's l is no longer read
    for (int i = threadIdx.x; i < nb * nz; i += blockDim.x)
      l[i] = ldp[((size_t)pv * npb + pb0) * nz + i];
    __syncthreads();
    for (int j = threadIdx.x; j < nb * ng; j += blockDim.x) {
      const int b = j / ng, g = j % ng;
      const R* row = Wk + (size_t)g * ldw;
      const R* lb = l + b * nz;
      R d = R(0);
      for (int z = 0; z < nz; ++z) d += row[z] * lb[z];
      ldm[((size_t)pv * npb + pb0 + b) * ng + g] = d;
    }
  }
}

// Blocks per pv of the LD-means kernel: the 2D table (mode 2) is costly FP64
// work (GB300's FP64 rate is 1/64 of FP32), built once per block, so all of a
// pv's passbands share one block; the 3D slab is a cheap lerp.
static dim3 ldm_grid(int npv, int npb, int mode) {
  const int ngroups = (npb + LDM_PBB - 1) / LDM_PBB;
  const int want = (mode == 2) ? 1 : (4096 + npv - 1) / npv;
  return dim3(npv, (unsigned)std::max(1, std::min(ngroups, want)));
}

// Dynamic shared memory of ldm_kernel<R>; above the default 48 KB (large ng)
// the kernel is opted in to the larger carve-out first.
template <typename R>
static size_t ldm_smem_bytes(int ng, int nz) {
  const size_t scratch = (sizeof(R) == 8) ? 0 : sizeof(double) * LDM_SCRATCH;
  const size_t bytes = ldm_scratch_offset<R>(ng, nz) + scratch;
  if (bytes > 48 * 1024)
    cudaFuncSetAttribute(ldm_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return bytes;
}

// Host launchers of the LD-means kernel for the other translation units.
template <typename R>
static void launch_ldm_impl(const R* ldp, int npv, int npb, int nz, const double* kw, int kw_stride, const R* W,
                            int nk, int ng, double dk, double kmin, double kmax, const double* ze, int mode,
                            const double* kmax_pv, R* ldm, cudaStream_t s) {
  ldm_kernel<R><<<ldm_grid(npv, npb, mode), 128, ldm_smem_bytes<R>(ng, nz), s>>>(
      ldp, npb, nz, kw, kw_stride, W, nk, ng, dk, kmin, kmax, ze, mode, kmax_pv, ldm);
}
void launch_ldm_f32(const float* ldp, int npv, int npb, int nz, const double* kw, int kw_stride, const float* W,
                    int nk, int ng, double dk, double kmin, double kmax, const double* ze, int mode,
                    const double* kmax_pv, float* ldm, cudaStream_t s) {
  launch_ldm_impl<float>(ldp, npv, npb, nz, kw, kw_stride, W, nk, ng, dk, kmin, kmax, ze, mode, kmax_pv, ldm, s);
}
void launch_ldm_f64(const double* ldp, int npv, int npb, int nz, const double* kw, int kw_stride, const double* W,
                    int nk, int ng, double dk, double kmin, double kmax, const double* ze, int mode,
                    const double* kmax_pv, double* ldm, cudaStream_t s) {
  launch_ldm_impl<double>(ldp, npv, npb, nz, kw, kw_stride, W, nk, ng, dk, kmin, kmax, ze, mode, kmax_pv, ldm, s);
}

// ---------------------------------------------------------------------------
// Basis tables of an affine law: B[ik][b][g] = sum_z W[ik][g][z] phi_b(mu_z),
// one thread per (ik, g), FP64 (and an FP32 copy).
// ---------------------------------------------------------------------------
__global__ void basis_tables_kernel(int law, int nb, const double* __restrict__ mu, int nz,
                                    const double* __restrict__ W, int nk, int ng, double* __restrict__ B64,
                                    float* __restrict__ B32) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nk * ng) return;
  const int ik = row / ng, g = row % ng;
  const double* w = W + (size_t)row * nz;
  for (int b = 0; b < nb; ++b) {
    double acc = 0.0;
    for (int z = 0; z < nz; ++z) acc += w[z] * basis_value(law, b, mu[z]);
    const size_t o = ((size_t)ik * nb + b) * ng + g;
    B64[o] = acc;
    if (B32) B32[o] = (float)acc;
  }
}

// LD means of an affine law from the basis tables, one block per pv:
//   ldm[pv, pb, g] = sum_b coef_b(pv, pb) ((1-ak) B[ik][b][g] + ak B[ik+1][b][g]),
// k, ik, ak as model_full.py:46-51.  Outside the 3D table (k outside
// [kmin, kmax], or ik+1 == nk) the 2D table at k is built row by row in FP64
// and applied to ldp, as the generic kernel does.
constexpr int MAX_BASIS = 16;

// Row g of the LD means of one pv for every passband from the 2D weight table
// built at k in FP64 (calculate_weights_2d, common.py:153-185): the k-outside-
// the-tables case of the affine-law kernels.  ldp_pv = the pv's [npb][nz]
// profiles, out = its [npb][ng] means.
template <typename R>
__device__ inline void ldm_direct_g(double k, int g, int ng, int nz, const double* __restrict__ ze,
                                    const R* ldp_pv, int npb, R* out) {
  const double gstep = (1.0 - 1e-7) / (double)(ng - 1);
  double gg = (double)g * gstep;
  if (g == ng - 1) gg = 1.0 - 1e-7;
  const double bb = gg * (1.0 + k);
  double w[64];
  double a0 = cci_acos(ze[0], k, bb), s = a0;
  w[0] = a0;
  for (int z = 1; z < nz; ++z) {
    const double a1 = cci_acos(ze[z], k, bb);
    w[z] = a1 - a0;
    a0 = a1;
    s += w[z];
  }
  for (int pb = 0; pb < npb; ++pb) {
    const R* l = ldp_pv + (size_t)pb * nz;
    double acc = 0.0;
    for (int z = 0; z < nz; ++z) acc += (w[z] / s) * (double)l[z];
    out[(size_t)pb * ng + g] = (R)acc;
  }
}

template <typename R>
__global__ void __launch_bounds__(128)
ldm_basis_kernel(int law, const double* __restrict__ ldc, int npar, int npb, const double* __restrict__ kw,
                 int kw_stride, const R* __restrict__ B, int nb, int nk, int ng, double dk, double kmin,
                 double kmax, const R* __restrict__ ldp, int nz, const double* __restrict__ ze,
                 R* __restrict__ ldm) {
  extern __shared__ __align__(16) unsigned char bsm[];
  R* coef = reinterpret_cast<R*>(bsm);                    // [npb][nb]
  __shared__ int s_ik;
  __shared__ double s_ak;
  const int pv = blockIdx.x;
  if (threadIdx.x == 0) {
    const double k = kw[(size_t)pv * kw_stride];
    int ik = -1;
    double ak = 0.0;
    if (kmin <= k && k <= kmax) {
      ik = (int)floor((k - kmin) / dk);
      ak = (k - kmin - ik * dk) / dk;
      if (ik + 1 >= nk || ik < 0) ik = -1;
    }
    s_ik = ik;
    s_ak = ak;
  }
  for (int pb = threadIdx.x; pb < npb; pb += blockDim.x) {
    double c[MAX_BASIS];
    basis_coefs(law, ldc + ((size_t)pv * npb + pb) * npar, npar, c);
    for (int b = 0; b < nb; ++b) coef[pb * nb + b] = (R)c[b];
  }
  __syncthreads();
  const int ik = s_ik;
  R* out = ldm + (size_t)pv * npb * ng;
  if (ik >= 0) {
    const R a1 = (R)s_ak, a0 = R(1) - (R)s_ak;
    const R* B0 = B + (size_t)ik * nb * ng;
    const R* B1 = B0 + (size_t)nb * ng;
    for (int j = threadIdx.x; j < npb * ng; j += blockDim.x) {
      const int pb = j / ng, g = j % ng;
      R d0 = R(0), d1 = R(0);
      for (int b = 0; b < nb; ++b) {
        d0 += coef[pb * nb + b] * __ldg(B0 + b * ng + g);
        d1 += coef[pb * nb + b] * __ldg(B1 + b * ng + g);
      }
      out[j] = a0 * d0 + a1 * d1;
    }
  } else {
    const double k = kw[(size_t)pv * kw_stride];
    for (int g = threadIdx.x; g < ng; g += blockDim.x)
      ldm_direct_g(k, g, ng, nz, ze, ldp + (size_t)pv * npb * nz, npb, out);
  }
}

// ---------------------------------------------------------------------------
// Orbit prologue, model_full.py:39-42 and 56-71, one thread per pv:
// validity, Taylor coefficients (solve2d), contact points (bounding_box).
// ---------------------------------------------------------------------------
struct OrbitArgs {
  const double *k, *t0, *p, *a, *inc, *e, *w, *exptimes;
  const int32_t *pbids, *epids, *nsamples;
  int nkc, ldt0, nep, npv, nlc, npb, nz;
  const void* ldp;       // validity probe ldp[pv, 0, 0] (double or float)
  int ldp_is_f32;
  // plain FP64 path
  double* orb64;
  // split path
  float *orb32, *lc32;
  const float* istar32;
  double t_ref, t_absmax;
  // split path with the LD profile evaluated here rather than read from
  // ldp / istar32 (the fused prologue): the law's coefficients ldc[npv, npb,
  // npar] and the mu grid, taken as FP32 as ld_tables_kernel<float> takes them
  int ld_direct, law, npar;
  const double *ldc, *mu;
};

constexpr int ORB_MAX_LDPAR = 4;   // coefficients per passband of the fused prologue's laws

// FP32 coefficients of (pv, pb), as ld_tables_kernel<float> converts them.
__device__ inline void ld_coefs_f32(const OrbitArgs& A, int pv, int pb, float* c) {
  const double* src = A.ldc + ((size_t)pv * A.npb + pb) * A.npar;
#pragma unroll
  for (int i = 0; i < ORB_MAX_LDPAR; ++i) c[i] = i < A.npar ? (float)src[i] : 0.0f;
}

// Plain FP64 path: validity, the FP64 Taylor coefficients and the contact
// times of one pv.
__device__ __forceinline__ void orbit_pv_f64(const OrbitArgs& A, int pv) {
  const double a = A.a[pv], e = A.e[pv], p = A.p[pv];
  const bool ldbad = A.ldp_is_f32 ? isnan(((const float*)A.ldp)[(size_t)pv * A.npb * A.nz])
                                  : isnan(((const double*)A.ldp)[(size_t)pv * A.npb * A.nz]);
  const bool valid = !(isnan(a) || a <= 1.0 || e < 0.0 || ldbad);
  double c[10];
  double t1 = 0.0, t4 = 0.0;
  const double k0 = A.k[(size_t)pv * A.nkc];
  if (valid) {
    solve2d_conj(p, a, A.inc[pv], e, A.w[pv], c);
    t1 = contact_point(k0, 1, c);
    t4 = contact_point(k0, 4, c);
  } else {
    for (int i = 0; i < 10; ++i) c[i] = 0.0;
  }
  double* o = A.orb64 + (size_t)pv * ORB64;
  for (int i = 0; i < 10; ++i) o[i] = c[i];
  o[10] = t1;
  o[11] = t4;
  o[12] = valid ? 1.0 : 0.0;
}

// Split path: the FP32 orbit record [ORB32] and the per-light-curve records
// [nlc][LC32] of one pv.  The pointers are restrict-qualified locals and the
// light curves go in groups of four with every load of a group issued before
// its records are stored, so the dependent loads (epoch id -> zero epoch,
// passband id -> coefficients) of different light curves overlap; both
// contact points are bisected in one loop; records are written 16 bytes at a
// time.
constexpr int ORB_LCG = 2;   // light curves per load group

__device__ __forceinline__ void orbit_pv_split(const OrbitArgs& A, int pv) {
  const double* __restrict__ t0v = A.t0 + (size_t)pv * A.ldt0;
  const double* __restrict__ kv = A.k + (size_t)pv * A.nkc;
  const double* __restrict__ exptimes = A.exptimes;
  const int32_t* __restrict__ epids = A.epids;
  const int32_t* __restrict__ pbids = A.pbids;
  const int32_t* __restrict__ nsamples = A.nsamples;
  float4* __restrict__ o4 = reinterpret_cast<float4*>(A.orb32 + (size_t)pv * ORB32);
  float4* __restrict__ q4 = reinterpret_cast<float4*>(A.lc32 + (size_t)pv * A.nlc * LC32);
  const double a = A.a[pv], e = A.e[pv], p = A.p[pv], inc = A.inc[pv], w = A.w[pv];
  const double k0 = kv[0];
  bool ldbad;
  if (A.ld_direct) {
    float c[ORB_MAX_LDPAR];
    ld_coefs_f32(A, pv, 0, c);
    ldbad = isnan(ld_value<float>(A.law, (float)A.mu[0], c, A.npar));
  } else {
    ldbad = isnan(((const float*)A.ldp)[(size_t)pv * A.npb * A.nz]);
  }
  double d0max = 0.0;
  for (int ep = 0; ep < A.nep; ++ep) d0max = fmax(d0max, fabs(t0v[ep] - A.t_ref));
  const bool valid = !(isnan(a) || a <= 1.0 || e < 0.0 || ldbad);
  float cf[10];
  float t1 = 0.0f, t4 = 0.0f;
  if (valid) {
    solve2d_conj_f32(p, a, inc, e, w, cf);
    contact_points14_f32((float)k0, cf, t1, t4);
  } else {
    for (int i = 0; i < 10; ++i) cf[i] = 0.0f;
  }
  const float p_hi = __double2float_rn(p);
  const float p_lo = __double2float_rn(p - (double)p_hi);
  // Bound of |fast-test tc - true tc|: 2^-24 (4 (T + |d0|) + 2 p), doubled.
  const double err = ldexp(1.0, -21) * (A.t_absmax + d0max + p) + 1e-9;
  int flags = valid ? FLAG_VALID : 0;
  for (int lc0 = 0; lc0 < A.nlc; lc0 += ORB_LCG) {
    double d0[ORB_LCG], kk[ORB_LCG], ex[ORB_LCG];
    int pb[ORB_LCG], ns[ORB_LCG];
    float is[ORB_LCG];
#pragma unroll
    for (int j = 0; j < ORB_LCG; ++j) {
      const int lc = min(lc0 + j, A.nlc - 1);
      pb[j] = pbids[lc];
      ns[j] = nsamples[lc];
      ex[j] = exptimes[lc];
      d0[j] = t0v[epids[lc]] - A.t_ref;
      kk[j] = kv[A.nkc == A.npb ? pb[j] : 0];
      // a non-finite disk integral makes every in-box point NaN, as (istar - I A)/istar does
      if (A.ld_direct) {
        float c[ORB_MAX_LDPAR];
        ld_coefs_f32(A, pv, pb[j], c);
        ld_integral<float>(A.law, c, is[j]);
      } else {
        is[j] = A.istar32[(size_t)pv * A.npb + pb[j]];
      }
    }
#pragma unroll
    for (int j = 0; j < ORB_LCG; ++j) {
      const int lc = lc0 + j;
      if (lc >= A.nlc) break;
      const double pad = 0.003 + ex[j];
      const double lo = (double)t1 - pad, hi = (double)t4 + pad;
      if (hi + 2 * err >= 0.5 * p || lo - 2 * err <= -0.5 * p) flags |= FLAG_WIDE;
      const float d0h = __double2float_rn(d0[j]);
      const float kf = (float)kk[j];
      float4* q = q4 + (size_t)lc * (LC32 / 4);
      // LC_FLO, LC_FHI, LC_D0H, LC_D0L | LC_LO, LC_HI, LC_K, LC_INV1PK | LC_INVIS, LC_EXPT, LC_INVNS, LC_NS | LC_PB
      q[0] = make_float4((float)(lo - err), (float)(hi + err), d0h, __double2float_rn(d0[j] - (double)d0h));
      q[1] = make_float4((float)lo, (float)hi, kf, 1.0f / (1.0f + kf));
      q[2] = make_float4(isfinite(is[j]) ? 1.0f / is[j] : __int_as_float(0x7fc00000), (float)ex[j],
                         1.0f / (float)ns[j], __int_as_float(ns[j]));
      q[3] = make_float4(__int_as_float(pb[j]), 0.0f, 0.0f, 0.0f);
    }
  }
  o4[0] = make_float4(cf[0], cf[1], cf[2], cf[3]);
  o4[1] = make_float4(cf[4], cf[5], cf[6], cf[7]);
  o4[2] = make_float4(cf[8], cf[9], p_hi, p_lo);
  o4[3] = make_float4(1.0f / p_hi, (float)err, __int_as_float(flags), 0.0f);
}

template <bool SPLIT>
__device__ __forceinline__ void orbit_pv(const OrbitArgs& A, int pv) {
  if (SPLIT)
    orbit_pv_split(A, pv);
  else
    orbit_pv_f64(A, pv);
}

template <bool SPLIT>
__global__ void orbit_kernel(OrbitArgs A) {
  const int pv = blockIdx.x * blockDim.x + threadIdx.x;
  if (pv < A.npv) orbit_pv<SPLIT>(A, pv);
}

// ---------------------------------------------------------------------------
// Fused split prologue for the affine laws with an analytic disk integral
// (uniform, linear, quadratic, quadratic-tri): one launch does the work of
// ld_tables_kernel<float>, ldm_basis_kernel<float> and orbit_kernel<true>
// (rrmodel.py:212-227 and model_full.py:39-71).
//   blocks [0, norb): orbit blocks.  Their first warp takes 32 pvs, one per
//     lane: the FP64 orbit chain is latency-bound, so it is spread thin, and
//     the lane evaluates the disk integral and the profile's validity probe
//     itself instead of waiting for the LD tables.
//   blocks [norb, ...): LD blocks, one warp per pv: the profile on the mu
//     grid and its disk integral (written out as ld_tables_kernel<float> does),
//     then the LD means from the basis tables, in FP32 (FP64 only for a pv
//     whose k lies outside the tables).
// The orbit blocks come first in the grid, so their chains start at once and
// the LD blocks fill the SMs around them.
// ---------------------------------------------------------------------------
constexpr int PRO_THREADS = 128;
constexpr int PRO_WARPS = PRO_THREADS / 32;
constexpr int PRO_MAX_COEF = 128;   // npb * npar and npb * nb floats staged per warp

struct ProArgs {
  OrbitArgs orb;
  int npv, npb, npar, nz, nb, nk, ng, law, kw_stride;
  const double *ldc, *mu, *kw, *ze;
  double kmin, kmax, dk, inv_dk;
  const float* B;
  float *ldp, *istar, *ldm;
};

// Basis coefficients of one passband from its FP32 coefficients
// (basis_coefs on the FP32 values).
__device__ inline void basis_coefs_f32(int law, const float* c, int npar, float* coef) {
  switch (law) {
    case LD_QUADRATIC_TRI: {
      const float a = sqrtf(c[0]), b = 2.0f * c[1];
      coef[0] = 1.0f; coef[1] = a * b; coef[2] = a * (1.0f - b);
      return;
    }
    default:
      coef[0] = 1.0f;
      for (int i = 1; i < basis_count(law, npar); ++i) coef[i] = c[i - 1];
  }
}

template <int LAW>
__global__ void __launch_bounds__(PRO_THREADS, 8) prologue_split_kernel(ProArgs P, int norb) {
  constexpr int NB = LAW == LD_UNIFORM ? 1 : (LAW == LD_LINEAR ? 2 : 3);   // basis_count of the law
  __shared__ float s_mu[MAX_NZ];
  __shared__ float s_c[PRO_WARPS][PRO_MAX_COEF];
  __shared__ float s_coef[PRO_WARPS][PRO_MAX_COEF];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if ((int)blockIdx.x < norb) {
    if (warp != 0) return;
    const int pv = blockIdx.x * 32 + lane;
    if (pv < P.npv) orbit_pv<true>(P.orb, pv);
    return;
  }
  for (int i = threadIdx.x; i < P.nz; i += PRO_THREADS) s_mu[i] = (float)P.mu[i];
  __syncthreads();
  const int pv = ((int)blockIdx.x - norb) * PRO_WARPS + warp;
  if (pv >= P.npv) return;   // warp-uniform; no block barrier follows
  const int npb = P.npb, npar = P.npar, nz = P.nz, ng = P.ng;
  float* sc = s_c[warp];
  float* scf = s_coef[warp];
  for (int i = lane; i < npb * npar; i += 32) sc[i] = (float)P.ldc[(size_t)pv * npb * npar + i];
  __syncwarp();
  // the profile and its disk integral (ld_tables_kernel<float>), lanes over the mu grid
  float* ldp_pv = P.ldp + (size_t)pv * npb * nz;
  for (int pb = 0; pb < npb; ++pb)
    for (int z = lane; z < nz; z += 32) ldp_pv[pb * nz + z] = ld_value<float>(LAW, s_mu[z], sc + pb * npar, npar);
  for (int pb = lane; pb < npb; pb += 32) {
    float is;
    ld_integral<float>(LAW, sc + pb * npar, is);
    P.istar[(size_t)pv * npb + pb] = is;
    basis_coefs_f32(LAW, sc + pb * npar, npar, scf + pb * NB);
  }
  __syncwarp();
  // the LD means (ldm_basis_kernel): per grid column g the two k rows' basis
  // columns are blended once, e_b = (1 - ak) B[ik][b][g] + ak B[ik+1][b][g],
  // then each passband is an NB-term dot product with its coefficients
  float* out = P.ldm + (size_t)pv * npb * ng;
  const double k = P.kw[(size_t)pv * P.kw_stride];
  int ik = -1;
  float a1 = 0.0f;
  if (P.kmin <= k && k <= P.kmax) {
    const double t = (k - P.kmin) * P.inv_dk;
    const double fl = floor(t);
    ik = (int)fl;
    a1 = (float)(t - fl);
    if (ik + 1 >= P.nk || ik < 0) ik = -1;
  }
  if (ik >= 0) {
    const float a0 = 1.0f - a1;
    const float* B0 = P.B + (size_t)ik * NB * ng;
    const float* B1 = B0 + (size_t)NB * ng;
    for (int g = lane; g < ng; g += 32) {
      float eb[NB];
#pragma unroll
      for (int b = 0; b < NB; ++b) eb[b] = a0 * __ldg(B0 + b * ng + g) + a1 * __ldg(B1 + b * ng + g);
      for (int pb = 0; pb < npb; ++pb) {
        float d = 0.0f;
#pragma unroll
        for (int b = 0; b < NB; ++b) d = fmaf(scf[pb * NB + b], eb[b], d);
        out[(size_t)pb * ng + g] = d;
      }
    }
  } else {
    for (int g = lane; g < ng; g += 32) ldm_direct_g(k, g, ng, nz, P.ze, (const float*)ldp_pv, npb, out);
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

// The flux of one point of a valid pv, with the reference's FP64 arithmetic
// (model_full.py:84-99): fold, box test, samples.
__device__ __forceinline__ double f64_point(const FluxF64Args& A, int pv, int pt, const double* o) {
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
  if (!(lo <= tc && tc <= hi)) return 1.0;
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
  return f / ns;
}

// The plain FP64 flux: one thread per point, every point through the
// reference's arithmetic.
__global__ void __launch_bounds__(256) flux_f64_kernel(FluxF64Args A) {
  const int pv = block_pv();
  const int pt = blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= A.npt || pv >= A.npv) return;
  const double* o = A.orb64 + (size_t)pv * ORB64;
  A.flux[(size_t)pv * A.ldflux + pt] = o[12] == 0.0 ? CUDART_NAN : f64_point(A, pv, pt, o);
}

// The FP64 flux with the fold done once per 128-point tile for the tiles that
// reach no box.  The reference's epoch floor(((t - t0) + p/2) / p) and
// tc = t - (t0 + epoch p), each step rounded as in f64_point, are
// non-decreasing in t.  So when a tile of one light curve has the same epoch
// at its earliest and latest time (tiles64: the FP64 summaries of
// rr_time_tiles_f64), every point of it has that epoch and a tc between the
// two ends' tc.  If that range misses the box, every point takes the
// reference's out-of-box value 1.0, and the tile is written without per-point
// work: the same bits as flux_f64_kernel, for ~1/60 of its FP64 instructions
// on the C1 workload.  A warp tests 32 tiles at once (one per lane) and
// writes the culled ones first; the others take f64_point, a lane per point.
constexpr int F64_WARPS = 4;

__global__ void __launch_bounds__(F64_WARPS * 32) flux_f64_culled_kernel(FluxF64Args A, const double* tiles64) {
  const int pv = block_pv();
  if (pv >= A.npv) return;   // block-uniform
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = (A.npt + TIME_TILE - 1) / TIME_TILE;
  const int tbase = (blockIdx.x * F64_WARPS + warp) * 32;
  if (tbase >= ntiles) return;   // warp-uniform
  const unsigned FULL = 0xffffffffu;
  const double* o = A.orb64 + (size_t)pv * ORB64;
  double* row = A.flux + (size_t)pv * A.ldflux;
  const bool valid = o[12] != 0.0;
  const int tile = tbase + lane;
  bool cull = !valid;
  if (valid && tile < ntiles) {
    const double tmin = tiles64[4 * (size_t)tile], tmax = tiles64[4 * (size_t)tile + 1];
    const int lc = (int)tiles64[4 * (size_t)tile + 2];
    if (lc >= 0) {
      const double t0 = A.t0[(size_t)pv * A.ldt0 + A.epids[lc]];
      const double p = A.p[pv];
      const double e0 = floor(__ddiv_rn(__dadd_rn(__dsub_rn(tmin, t0), __dmul_rn(0.5, p)), p));
      const double e1 = floor(__ddiv_rn(__dadd_rn(__dsub_rn(tmax, t0), __dmul_rn(0.5, p)), p));
      if (e0 == e1) {
        const double c = __dadd_rn(t0, __dmul_rn(e0, p));
        const double tc0 = __dsub_rn(tmin, c), tc1 = __dsub_rn(tmax, c);
        const double pad = __dadd_rn(0.003, A.exptimes[lc]);
        const double lo = __dsub_rn(o[10], pad), hi = __dadd_rn(o[11], pad);
        cull = tc1 < lo || tc0 > hi;
      }
    }
  }
  const int jn = min(32, ntiles - tbase);
  const unsigned jmask = jn == 32 ? FULL : (1u << jn) - 1u;
  const unsigned cmask = __ballot_sync(FULL, cull) & jmask;
  const double fill = valid ? 1.0 : CUDART_NAN;
  const bool vec = ((A.ldflux & 1) == 0) && ((reinterpret_cast<uintptr_t>(A.flux) & 15) == 0);
  for (unsigned m = cmask; m; m &= m - 1u) {
    const int p0 = (tbase + __ffs(m) - 1) * TIME_TILE;
    if (vec && p0 + TIME_TILE <= A.npt) {
      double2* q = reinterpret_cast<double2*>(row + p0) + 2 * lane;
      __stcs(q, make_double2(fill, fill));
      __stcs(q + 1, make_double2(fill, fill));
    } else {
      for (int q = 0; q < 4; ++q)
        if (p0 + 32 * q + lane < A.npt) row[p0 + 32 * q + lane] = fill;
    }
  }
  for (unsigned m = ~cmask & jmask; m; m &= m - 1u) {
    const int p0 = (tbase + __ffs(m) - 1) * TIME_TILE;
    for (int q = 0; q < 4; ++q) {
      const int pt = p0 + 32 * q + lane;
      if (pt < A.npt) row[pt] = f64_point(A, pv, pt, o);
    }
  }
}

// ---------------------------------------------------------------------------
// Split-precision flux.  The output row of a pv is cut into warp tiles of
// 128 consecutive points.  A block stages the pv's orbit record and its
// per-light-curve records in shared memory, so the per-point work has no
// dependent global loads, and its warps take a range of tiles.  A warp tests
// 32 of its tiles at once against the precomputed tile summaries (one lane
// per tile): a tile of one light curve whose time range misses every box
// copy is one 16-byte store of ones per lane.  The other tiles load their
// FP32-pair times (slot q of lane l holds point q * 32 + l) and take the
// per-point path: the phase-folded time exact in FP32 pairs (error-free
// transformations) and the box test; then, in FP32, z, the LD-table lerp and
// the kite area on the limb, or, with several samples per point, a per-warp
// list of (point, sample) pairs spread over the lanes and summed with a
// segmented shuffle reduction.  Output F = 1 - deficit.
// ---------------------------------------------------------------------------
constexpr int SPLIT_WARPS = 8;                // warps per block of the serving kernel
constexpr int SPLIT_PTS = 4;                 // points per lane
constexpr int WARP_TILE = 32 * SPLIT_PTS;    // points per warp tile

struct FluxSplitArgs {
  const float2* times_ff;
  const int32_t* lcids;
  const float *orb32, *lc32, *ldm;
  int npt, npv, npb, nlc, ng, ldflux;
  float inv_dg;
  void* flux;          // float or double rows (the kernel's OutT)
  int transits_only;   // store only the tiles that reach a transit (and invalid rows); the rest holds 1
};

// Output rows of the split flux kernels: FP32 (the split path's own type), or
// FP64 (the reference's output type, each FP32 result widened exactly).  A
// culled tile is one 16-byte store of the fill value per lane (FP32) or two
// (FP64).
template <typename OutT>
struct TileOut;

template <>
struct TileOut<float> {
  static __device__ __forceinline__ void fill(float* row, int tile, int lane, float v) {
    __stcs(reinterpret_cast<float4*>(row) + lane + (size_t)tile * (32 * 4 / 4), make_float4(v, v, v, v));
  }
};

template <>
struct TileOut<double> {
  static __device__ __forceinline__ void fill(double* row, int tile, int lane, float v) {
    const double d = v;
    double2* q = reinterpret_cast<double2*>(row) + (size_t)tile * 64 + 2 * lane;
    __stcs(q, make_double2(d, d));
    __stcs(q + 1, make_double2(d, d));
  }
};

constexpr int LC_SMEM = 64;                  // light-curve records staged in shared memory

struct WarpList {
  float tc[WARP_TILE];
  int lc[WARP_TILE];
  int off[WARP_TILE + 1];
  float acc[WARP_TILE];
};

// Per-point path for one warp tile of one pv (slot q of lane l = the tile's
// point q * 32 + l).  Phase-folded times: for a tile of one light curve whose
// span plus box half-width is below p/2, the exact time of the tile's first
// point plus each point's (exact, small) offset from it; otherwise a fast
// FP32 test per point and the exact reduction for candidates.  Then the
// samples of the in-box points: with one sample per point, per point in
// place, skipping slots without an in-box point as a whole warp; else a
// per-warp list whose (point, sample) pairs are spread over the lanes and
// summed with a segmented shuffle reduction.  res[] holds 1.0 on entry and
// the flux of in-box points on exit.
__device__ __forceinline__ void split_tile_points(const float* __restrict__ orb, const float* __restrict__ LCR,
                                                  const float* __restrict__ ldm_pv, int ng, float inv_dg,
                                                  bool wide, float4 tm, const float* hi, const float* lo,
                                                  const int* lcv, WarpList& L, int lane, float* res) {
  const unsigned FULL = 0xffffffffu;
  const float p_hi = orb[10], p_lo = orb[11], inv_p = orb[12];
  const int tlc = __float_as_int(tm.z);
  float tcq[SPLIT_PTS];
  unsigned inb = 0;
  // Tile-relative times are exact whenever no point of the tile can fold onto
  // another box copy: span + |box| < p/2 (points whose offset crosses p/2 are
  // then out of box in both foldings).
  const float* RT = LCR + (tlc >= 0 ? tlc : 0) * LC32;
  if (!wide && tlc >= 0 && (tm.y - tm.x) + fmaxf(-RT[LC_LO], RT[LC_HI]) < 0.5f * p_hi) {
    const float* R = RT;
    const float h0 = __shfl_sync(FULL, hi[0], 0), l0 = __shfl_sync(FULL, lo[0], 0);
    const float n0 = floorf(fmaf(h0 - R[LC_D0H], inv_p, 0.5f));
    float tail0;
    const float s0 = exact_tc_pair(h0, l0, R[LC_D0H], R[LC_D0L], n0, p_hi, p_lo, tail0);
    const float blo = R[LC_LO], bhi = R[LC_HI];
#pragma unroll
    for (int q = 0; q < SPLIT_PTS; ++q) {
      // s0 + (hi - h0) is exact (Sterbenz) near the transit, where the two
      // nearly cancel; the small terms go in last: one rounding at |tc| scale
      tcq[q] = (s0 + (hi[q] - h0)) + ((lo[q] - l0) + tail0);
      if (lcv[q] >= 0 && blo <= tcq[q] && tcq[q] <= bhi) inb |= 1u << q;
    }
  } else {
#pragma unroll
    for (int q = 0; q < SPLIT_PTS; ++q) {
      tcq[q] = 0.0f;
      if (lcv[q] < 0) continue;
      const float4 f = *reinterpret_cast<const float4*>(LCR + lcv[q] * LC32);  // flo, fhi, d0h, d0l
      const float sv = hi[q] - f.z;
      const float n = floorf(fmaf(sv, inv_p, 0.5f));
      const float r = fmaf(-n, p_hi, sv);
      if (wide || (r >= f.x && r <= f.y)) {
        const float t = exact_tc(hi[q], lo[q], f.z, f.w, n, p_hi, p_lo);
        const float* R = LCR + lcv[q] * LC32;
        tcq[q] = t;
        if (R[LC_LO] <= t && t <= R[LC_HI]) inb |= 1u << q;
      }
    }
  }
  if (!__ballot_sync(FULL, inb != 0)) return;
  // Slot q of the lanes holds the tile's 32 consecutive points q*32 .. q*32+31:
  // a slot without an in-box point skips the per-point work as a whole warp.
  unsigned act = 0;
#pragma unroll
  for (int q = 0; q < SPLIT_PTS; ++q) act |= (__ballot_sync(FULL, inb >> q & 1u) ? 1u : 0u) << q;
  bool single;
  if (tlc >= 0) {
    single = __float_as_int(RT[LC_NS]) == 1;   // one light curve: warp-uniform
  } else {
    single = true;
#pragma unroll
    for (int q = 0; q < SPLIT_PTS; ++q)
      if (inb >> q & 1u) single = single && (__float_as_int(LCR[lcv[q] * LC32 + LC_NS]) == 1);
    single = __all_sync(FULL, single);
  }
  if (single) {
    // One sample per point.  A point whose planet disk is fully inside the
    // star (area pi k^2) is finished in place; points on the limb (kite area,
    // two atan2) are gathered into the warp's list and evaluated 32 at a time,
    // so that the costly branch runs with full lanes.
    unsigned limb = 0;
    float zq[SPLIT_PTS];
    if (tlc >= 0) {
      // one light curve in the tile: its record in registers, the orbit
      // polynomial from vector loads, z = r2 rsqrt(r2) (2 ulp)
      const float k = RT[LC_K], gsc = RT[LC_INV1PK] * inv_dg, invis = RT[LC_INVIS];
      const float* lda = ldm_pv + __float_as_int(RT[LC_PB]) * ng;
      const float lim_out = 1.0f + k, lim_in = (k < 1.0f) ? 1.0f - k : -1.0f;
      const float area_in = float(PI) * k * k * invis;
      const float4 ca = *reinterpret_cast<const float4*>(orb);
      const float4 cb = *reinterpret_cast<const float4*>(orb + 4);
      const float2 cc = *reinterpret_cast<const float2*>(orb + 8);
      // the active slots side by side, without per-lane branches until the
      // loads are issued, so that their dependent chains overlap
      float frq[SPLIT_PTS], l0q[SPLIT_PTS], l1q[SPLIT_PTS];
#pragma unroll
      for (int q = 0; q < SPLIT_PTS; ++q) {
        zq[q] = 0.0f;
        frq[q] = l0q[q] = l1q[q] = 0.0f;
        if (!(act >> q & 1u)) continue;   // warp-uniform
        const float t = tcq[q];
        const float x = fmaf(t, fmaf(t, fmaf(t, fmaf(t, cb.x, ca.w), ca.z), ca.y), ca.x);
        const float y = fmaf(t, fmaf(t, fmaf(t, fmaf(t, cc.y, cc.x), cb.w), cb.z), cb.y);
        const float r2 = fmaf(x, x, y * y);
        zq[q] = r2 > 0.0f ? r2 * rsqrtf(r2) : 0.0f;
        const float gg = fminf(zq[q], lim_out) * gsc;
        const int i = min(max((int)gg, 0), ng - 2);
        frq[q] = gg - (float)i;
        const bool need = (inb >> q & 1u) && zq[q] < lim_out;   // inner and limb points
        l0q[q] = need ? __ldg(lda + i) : 0.0f;
        l1q[q] = need ? __ldg(lda + i + 1) : 0.0f;
      }
      // classification by selects: no overlap (1 - 0 / istar, NaN with a NaN
      // istar), fully inside (the lerp times pi k^2 / istar) or on the limb
      const float res_out = 1.0f - 0.0f * invis;
#pragma unroll
      for (int q = 0; q < SPLIT_PTS; ++q) {
        if (!(act >> q & 1u)) continue;   // warp-uniform
        const bool in = inb >> q & 1u;
        const bool ovl = zq[q] < lim_out, inner = zq[q] <= lim_in;
        const float r_in = 1.0f - fmaf(frq[q], l1q[q] - l0q[q], l0q[q]) * area_in;
        res[q] = in ? (ovl ? (inner ? r_in : res[q]) : res_out) : res[q];
        limb |= (in && ovl && !inner) ? 1u << q : 0u;
      }
      // Limb points (kite area, two atan2) in place, slot by slot: the limb
      // points of a slot are consecutive in time (an ingress or an egress),
      // so one or two slots of a tile hold them all, and their table values
      // came with the loads above.  For k < 1 every limb point is in the kite
      // case, evaluated on all lanes of the slot without branches and kept
      // where the lane's point is on the limb.
#pragma unroll
      for (int q = 0; q < SPLIT_PTS; ++q) {
        if (!(act >> q & 1u)) continue;                    // warp-uniform
        if (!__ballot_sync(FULL, limb >> q & 1u)) continue;  // warp-uniform
        const bool lm = limb >> q & 1u;
        const float lerp = fmaf(frq[q], l1q[q] - l0q[q], l0q[q]);
        if (k <= 0.25f) {                                  // tile-uniform
          const float zz = lm ? zq[q] : 1.0f;              // an in-range z for the other lanes
          const float a = kite_star_f32_smallk(k, zz);
          res[q] = lm ? 1.0f - (lerp * a) * invis : res[q];
        } else if (k < 1.0f) {                             // tile-uniform
          const float zz = lm ? zq[q] : 1.0f;
          const float a = kite_star_f32(k, zz);
          res[q] = lm ? 1.0f - (lerp * a) * invis : res[q];
        } else if (lm) {
          float kap;
          res[q] = 1.0f - (lerp * ccia_star<float>(k, zq[q], kap)) * invis;
        }
      }
      return;
    } else {
#pragma unroll
      for (int q = 0; q < SPLIT_PTS; ++q) {
        zq[q] = 0.0f;
        if (!(inb >> q & 1u)) continue;
        const float* R = LCR + lcv[q] * LC32;
        const float k = R[LC_K];
        const float z = sep_c_f32(tcq[q], orb);
        zq[q] = z;
        if (!(z < 1.0f + k)) {                         // no overlap: 1 - 0 / istar (NaN with a NaN istar)
          res[q] = 1.0f - 0.0f * R[LC_INVIS];
          continue;
        }
        if (k < 1.0f && z <= 1.0f - k) {
          const float gg = z * R[LC_INV1PK] * inv_dg;
          int i = (int)gg;
          i = min(max(i, 0), ng - 2);
          const float fr = gg - (float)i;
          const float* lda = ldm_pv + __float_as_int(R[LC_PB]) * ng;
          const float l0 = __ldg(lda + i), l1 = __ldg(lda + i + 1);
          res[q] = 1.0f - fmaf(fr, l1 - l0, l0) * (float(PI) * k * k) * R[LC_INVIS];
        } else {
          limb |= 1u << q;
        }
      }
    }
    if (!__ballot_sync(FULL, limb != 0)) return;
    int nl = 0;
    int posq[SPLIT_PTS];
#pragma unroll
    for (int q = 0; q < SPLIT_PTS; ++q) {
      posq[q] = -1;
      if (!(act >> q & 1u)) continue;   // warp-uniform
      const bool in = limb >> q & 1u;
      const unsigned m = __ballot_sync(FULL, in);
      if (in) {
        const int pos = nl + __popc(m & ((1u << lane) - 1u));
        L.tc[pos] = zq[q];
        L.lc[pos] = lcv[q];
        posq[q] = pos;
      }
      nl += __popc(m);
    }
    __syncwarp();
    for (int i0 = 0; i0 < nl; i0 += 32) {
      const int it = i0 + lane;
      if (it < nl) {
        const float z = L.tc[it];
        const float* R = LCR + L.lc[it] * LC32;
        const float k = R[LC_K];
        const float gg = z * R[LC_INV1PK] * inv_dg;
        int i = (int)gg;
        i = min(max(i, 0), ng - 2);
        const float fr = gg - (float)i;
        const float* lda = ldm_pv + __float_as_int(R[LC_PB]) * ng;
        const float l0 = __ldg(lda + i), l1 = __ldg(lda + i + 1);
        float kap;
        L.acc[it] = fmaf(fr, l1 - l0, l0) * ccia_star<float>(k, z, kap);
      }
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < SPLIT_PTS; ++q)
      if (posq[q] >= 0) res[q] = 1.0f - L.acc[posq[q]] * LCR[lcv[q] * LC32 + LC_INVIS];
    __syncwarp();
    return;
  }
  int nitems = 0;
  int posq[SPLIT_PTS];
#pragma unroll
  for (int q = 0; q < SPLIT_PTS; ++q) {
    const bool in = inb >> q & 1u;
    const unsigned m = __ballot_sync(FULL, in);
    posq[q] = -1;
    if (in) {
      const int pos = nitems + __popc(m & ((1u << lane) - 1u));
      L.tc[pos] = tcq[q];
      L.lc[pos] = lcv[q];
      posq[q] = pos;
    }
    nitems += __popc(m);
  }
  __syncwarp();
  // exclusive prefix sum of the sample counts -> L.off
  int carry = 0;
  for (int c0 = 0; c0 < nitems; c0 += 32) {
    const int it = c0 + lane;
    const int v = (it < nitems) ? __float_as_int(LCR[L.lc[it] * LC32 + LC_NS]) : 0;
    int incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int u = __shfl_up_sync(FULL, incl, d);
      if (lane >= d) incl += u;
    }
    if (it < nitems) {
      L.off[it] = carry + incl - v;
      L.acc[it] = 0.0f;
    }
    carry += __shfl_sync(FULL, incl, 31);
  }
  __syncwarp();
  const int total = carry;
  for (int f0 = 0; f0 < total; f0 += 32) {
    const int f = f0 + lane;
    float d = 0.0f;
    int item = -1;
    if (f < total) {
      int lo_i = 0, hi_i = nitems - 1;   // largest item with off[item] <= f
      while (lo_i < hi_i) {
        const int mid = (lo_i + hi_i + 1) >> 1;
        if (L.off[mid] <= f) lo_i = mid; else hi_i = mid - 1;
      }
      item = lo_i;
      const int smp = f - L.off[item];
      const float* R = LCR + L.lc[item] * LC32;
      const float k = R[LC_K];
      // time_offset = exptime ((isample - 0.5)/ns - 0.5), isample = smp + 1
      const float t = L.tc[item] + R[LC_EXPT] * fmaf(float(smp) + 0.5f, R[LC_INVNS], -0.5f);
      const float z = sep_c_f32(t, orb);
      if (z < 1.0f + k) {
        const float gg = z * R[LC_INV1PK] * inv_dg;
        int i = (int)gg;
        i = min(max(i, 0), ng - 2);
        const float fr = gg - (float)i;
        const float* lda = ldm_pv + __float_as_int(R[LC_PB]) * ng;
        const float l0 = __ldg(lda + i), l1 = __ldg(lda + i + 1);
        float kap;
        d = fmaf(fr, l1 - l0, l0) * ccia_star<float>(k, z, kap);
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
#pragma unroll
  for (int q = 0; q < SPLIT_PTS; ++q) {
    if (posq[q] >= 0) {
      const float* R = LCR + lcv[q] * LC32;
      res[q] = 1.0f - L.acc[posq[q]] * R[LC_INVIS] * R[LC_INVNS];
    }
  }
  __syncwarp();
}

// One block's share of one parameter vector: stage the pv's orbit and
// light-curve records in shared memory, then the warps loop over the tiles
// t_first + warp, + t_step, ... below t_end, 32 at a time: the cull tests,
// the stores of the culled tiles (walking the set bits of the cull mask),
// then the per-point path of the others.  Ends without a barrier: the caller
// synchronises before staging another pv.
template <typename OutT>
__device__ __forceinline__ void split_pv_tiles(const FluxSplitArgs& A, int pv, int t_first, int t_step, int t_end,
                                               float* recs, bool lc_in_smem, WarpList* lists) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const float* lcg = A.lc32 + (size_t)pv * A.nlc * LC32;
  if (threadIdx.x < ORB32) recs[threadIdx.x] = __ldg(A.orb32 + (size_t)pv * ORB32 + threadIdx.x);
  if (lc_in_smem)
    for (int i = threadIdx.x; i < A.nlc * LC32; i += blockDim.x) recs[ORB32 + i] = __ldg(lcg + i);
  __syncthreads();
  const float* orb = recs;
  const float* LCR = lc_in_smem ? recs + ORB32 : lcg;
  const int flags = __float_as_int(orb[14]);
  const bool valid = flags & FLAG_VALID;
  const bool wide = flags & FLAG_WIDE;
  const float p_hi = orb[10], inv_p = orb[12];
  const float* ldm_pv = A.ldm + (size_t)pv * A.npb * A.ng;
  OutT* row = static_cast<OutT*>(A.flux) + (size_t)pv * A.ldflux;
  const bool row_vec = ((A.ldflux & 3) == 0) && ((reinterpret_cast<uintptr_t>(A.flux) & 15) == 0);
  const float4* meta = reinterpret_cast<const float4*>(reinterpret_cast<const float*>(A.times_ff) +
                                                       time_meta_offset(A.npt));
  WarpList& L = lists[warp];
  const unsigned FULL = 0xffffffffu;
  // The warp's tiles are t_first + warp + j t_step, j < ntl.  A culled tile is
  // one 16-byte store of the fill value per lane (ones; NaN for an invalid
  // pv, whose tiles are all "culled"); only the row's last tile can be
  // partial, and it is stored point by point.
  const int tw0 = t_first + warp;
  const int ntl = tw0 < t_end ? (t_end - tw0 + t_step - 1) / t_step : 0;
  const int tile_part = (A.npt % WARP_TILE) ? A.npt / WARP_TILE : -1;
  const float fill = valid ? 1.0f : __int_as_float(0x7fc00000);
  for (int j0 = 0; j0 < ntl; j0 += 32) {
    // The cull test of the warp's next 32 tiles, one tile per lane: the
    // tile's time range (from its summary) against the box copies around it,
    // the rounding of t - d0 and of j p covered by the error bound in the box
    // (flo, fhi).
    const int tl = tw0 + (j0 + lane) * t_step;
    bool cull = !valid;
    if (valid && !wide && j0 + lane < ntl) {
      const float4 tm = __ldg(meta + tl);
      const int tlc = __float_as_int(tm.z);
      if (tlc >= 0) {
        const float4 f = *reinterpret_cast<const float4*>(LCR + tlc * LC32);  // flo, fhi, d0h, d0l
        const float smin = tm.x - f.z, smax = tm.y - f.z;
        const float j0f = ceilf((smin - f.y) * inv_p);
        bool hit = false;
#pragma unroll
        for (int dj = -1; dj <= 1; ++dj) {
          const float jj = j0f + (float)dj;
          hit = hit || (fmaf(jj, p_hi, f.x) <= smax && fmaf(jj, p_hi, f.y) >= smin);
        }
        cull = !hit;
      }
    }
    const int jn = min(32, ntl - j0);
    const unsigned jmask = jn == 32 ? 0xffffffffu : (1u << jn) - 1u;
    const unsigned cmask = __ballot_sync(FULL, cull) & jmask;
    // the culled tiles first, walking the set bits of the mask (none when the
    // caller has already set the row to 1; an invalid pv's NaN always)
    for (unsigned m = (A.transits_only && valid) ? 0u : cmask; m; m &= m - 1u) {
      const int tile = tw0 + (j0 + __ffs(m) - 1) * t_step;
      if (row_vec && tile != tile_part) {
        TileOut<OutT>::fill(row, tile, lane, fill);
      } else {
        const int pt0 = tile * WARP_TILE + lane * SPLIT_PTS;
        for (int q = 0; q < SPLIT_PTS; ++q)
          if (pt0 + q < A.npt) __stcs(row + pt0 + q, (OutT)fill);
      }
    }
    // then the tiles that reach a box copy
    for (unsigned m = ~cmask & jmask; m; m &= m - 1u) {
      const int tile = tw0 + (j0 + __ffs(m) - 1) * t_step;
      // The tile reaches a box copy (the cull test above said so).  Slot q of
      // lane l holds point tile * 128 + q * 32 + l: each slot is 32
      // consecutive points, coalesced in its loads and stores.
      const float4 tm = __ldg(meta + tile);                 // tmin, tmax, lc
      const int ps0 = tile * WARP_TILE + lane;
      float res[SPLIT_PTS] = {1.0f, 1.0f, 1.0f, 1.0f};
      float hi[SPLIT_PTS], lo[SPLIT_PTS];
      int lcv[SPLIT_PTS];
#pragma unroll
      for (int q = 0; q < SPLIT_PTS; ++q) {
        const int pt = ps0 + 32 * q;
        if (pt < A.npt) {
          const float2 tt = __ldg(A.times_ff + pt);
          hi[q] = tt.x; lo[q] = tt.y; lcv[q] = __ldg(A.lcids + pt);
        } else {
          hi[q] = 0.0f; lo[q] = 0.0f; lcv[q] = -1;
        }
      }
      split_tile_points(orb, LCR, ldm_pv, A.ng, A.inv_dg, wide, tm, hi, lo, lcv, L, lane, res);
#pragma unroll
      for (int q = 0; q < SPLIT_PTS; ++q)
        if (ps0 + 32 * q < A.npt) __stcs(row + ps0 + 32 * q, (OutT)res[q]);
    }
  }
}

// Flux launch shape: blocks of FLUX_NW warps, each block one range of at
// most FLUX_CHUNK consecutive warp tiles of one pv (its warps interleaved over
// the range).  Grid: x = tile ranges, y/z = parameter vectors.  A small block
// gives its registers back as soon as its own tiles are done, so a range that
// holds a transit keeps no finished warps resident, and the hardware block
// scheduler balances the ranges over the SMs.  The pv's records are staged in
// dynamic shared memory sized to the light-curve count.
constexpr int FLUX_NW = 2;
constexpr int FLUX_CHUNK = 32;

template <bool LC_IN_SMEM, typename OutT>
__global__ void __launch_bounds__(FLUX_NW * 32) flux_split_kernel(FluxSplitArgs A, int chunk) {
  __shared__ WarpList lists[FLUX_NW];
  extern __shared__ __align__(16) float flux_recs[];
  const int pv = block_pv();
  if (pv >= A.npv) return;  // block-uniform
  const int ntiles = (A.npt + WARP_TILE - 1) / WARP_TILE;
  const int t0 = blockIdx.x * chunk;
  const int t1 = t0 + chunk < ntiles ? t0 + chunk : ntiles;
  split_pv_tiles<OutT>(A, pv, t0, FLUX_NW, t1, flux_recs, LC_IN_SMEM, lists);
}

// ---------------------------------------------------------------------------
// Serving: one persistent launch over the work items of many requests.  Each
// block takes the next item (request, pv range, tile range) from a device
// counter and runs split_pv_tiles for it with that request's tables; the
// item list is complete at launch, so no block ever waits for work.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(SPLIT_WARPS * 32, 3)
serve_split_kernel(const rr_serve_request* __restrict__ reqs, const rr_serve_item* __restrict__ items,
                   const int* __restrict__ nitems_p, int* __restrict__ counter) {
  // the per-warp lists of the RoadRunner tiles and the tile state of the
  // transmission-spectroscopy tiles share the block's shared memory
  __shared__ union ServeSmem {
    WarpList lists[SPLIT_WARPS];
    TsSmem<float> ts;
  } U;
  __shared__ __align__(16) float recs[ORB32 + LC_SMEM * LC32];
  __shared__ int s_item;
  const int nitems = *nitems_p;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
    __syncthreads();
    const int it = s_item;
    __syncthreads();
    if (it >= nitems) return;
    const rr_serve_item w = items[it];
    const rr_serve_request& r = reqs[w.req];
    if (r.kind == 1) {
      // transmission spectroscopy (rr_ts.cuh): items span at most 32 tiles
      TsArgs<float> T{};
      T.times_ff = reinterpret_cast<const float2*>(r.times_ff);
      T.orb = r.orb32; T.ch = r.lc32; T.ldm = r.ldm; T.flux = r.flux;
      T.ldflux = r.ldflux; T.npt = r.npt; T.npb = r.npb; T.ng = r.ng; T.nsamples0 = r.nsamples0;
      T.exptime0 = (double)r.exptime0; T.dg = r.dg;
      for (int pv = w.pv0; pv < w.pv1; ++pv) {
        __syncthreads();   // the previous pv's record is consumed
        if (threadIdx.x < TS_ORB) recs[threadIdx.x] = __ldg(r.orb32 + (size_t)pv * TS_ORB + threadIdx.x);
        __syncthreads();
        ts_range<float, true>(T, pv, w.tile0, w.tile1, recs, U.ts);
      }
      __syncthreads();
      continue;
    }
    WarpList* lists = U.lists;
    FluxSplitArgs A{};
    A.times_ff = reinterpret_cast<const float2*>(r.times_ff);
    A.lcids = r.lcids;
    A.orb32 = r.orb32; A.lc32 = r.lc32; A.ldm = r.ldm;
    A.npt = r.npt; A.npv = r.npv; A.npb = r.npb; A.nlc = r.nlc; A.ng = r.ng; A.ldflux = (int)r.ldflux;
    A.inv_dg = r.inv_dg; A.flux = r.flux;
    const bool lc_smem = r.nlc <= LC_SMEM;
    for (int pv = w.pv0; pv < w.pv1; ++pv) {
      split_pv_tiles<float>(A, pv, w.tile0, SPLIT_WARPS, w.tile1, recs, lc_smem, lists);
      __syncthreads();
    }
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
  (void)nep;
  Carve c(nullptr);
  c.take<float>((size_t)npv * ORB32);
  c.take<float>((size_t)npv * nlc * LC32);
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
  float *orb, *lc, *ldm;
};

static SplitTables carve_split(void* ws, int npv, int npb, int nlc, int ng) {
  Carve cv(ws);
  SplitTables t;
  t.orb = cv.take<float>((size_t)npv * ORB32);
  t.lc = cv.take<float>((size_t)npv * nlc * LC32);
  t.ldm = cv.take<float>((size_t)npv * npb * ng);
  return t;
}

int rr_prepare_f64(const double* k, int nkc, const double* p, const double* a, const double* inc,
                   const double* e, const double* w, int npv, int npb, const double* ldp,
                   const double* weights, int nk, int ng, int nz, double dk, double kmin, double kmax,
                   const double* z_edges, void* workspace, size_t workspace_bytes, void* stream,
                   int law, const double* ldc, int npar, const double* basis, int nb) {
  if (nkc > 1 && nkc != npb) return RR_ERR_SHAPE;
  if (npv < 0 || npb < 1 || nk < 2 || ng < 2 || nz < 1 || nz > MAX_NZ || nkc < 1) return RR_ERR_ARG;
  if (npv == 0) return RR_OK;
  if (workspace_bytes < rr_full_f64_workspace_bytes(npv, npb, ng)) return RR_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  Carve cv(workspace);
  double* orb = cv.take<double>((size_t)npv * ORB64);
  double* ldm = cv.take<double>((size_t)npv * npb * ng);
  if (basis && nb > 0 && nb <= MAX_BASIS && ldc) {
    ldm_basis_kernel<double><<<npv, 128, sizeof(double) * npb * nb, s>>>(
        law, ldc, npar, npb, k, nkc, basis, nb, nk, ng, dk, kmin, kmax, ldp, nz, z_edges, ldm);
  } else {
    ldm_kernel<double><<<ldm_grid(npv, npb, 0), 128, ldm_smem_bytes<double>(ng, nz), s>>>(
        ldp, npb, nz, k, nkc, weights, nk, ng, dk, kmin, kmax, z_edges, 0, nullptr, ldm);
  }
  OrbitArgs oa{};
  oa.k = k; oa.p = p; oa.a = a; oa.inc = inc; oa.e = e; oa.w = w;
  oa.nkc = nkc; oa.npv = npv; oa.npb = npb; oa.nz = nz;
  oa.ldp = ldp; oa.ldp_is_f32 = 0; oa.orb64 = orb;
  orbit_kernel<false><<<(npv + 31) / 32, 32, 0, s>>>(oa);
  return check_launch("rr_prepare_f64");
}

int rr_flux_f64_range(const double* times, int npt, const double* k, int nkc, const double* t0, int ldt0,
                      const double* p, int npv, int nlc, int npb, const int32_t* lcids, const int32_t* pbids,
                      const int32_t* epids, const int32_t* nsamples, const double* exptimes,
                      const double* istar, int ng, double dg, const void* workspace, int pv0, int pv1,
                      double* flux, int ldflux, void* stream) {
  if (nkc > 1 && nkc != npb) return RR_ERR_SHAPE;
  if (npt < 0 || npv < 0 || nlc < 1 || npb < 1 || ng < 2 || nkc < 1 || ldflux < npt) return RR_ERR_ARG;
  if (pv0 < 0 || pv1 > npv || pv0 > pv1) return RR_ERR_ARG;
  if (pv1 == pv0 || npt == 0) return RR_OK;
  Carve cv(const_cast<void*>(workspace));
  double* orb = cv.take<double>((size_t)npv * ORB64);
  double* ldm = cv.take<double>((size_t)npv * npb * ng);
  // the range's parameters and records: the kernel indexes pv from 0 within it
  FluxF64Args fa{};
  fa.times = times; fa.k = k + (size_t)pv0 * nkc; fa.t0 = t0 + (size_t)pv0 * ldt0; fa.p = p + pv0;
  fa.exptimes = exptimes; fa.istar = istar + (size_t)pv0 * npb;
  fa.ldm = ldm + (size_t)pv0 * npb * ng; fa.orb64 = orb + (size_t)pv0 * ORB64;
  fa.lcids = lcids; fa.pbids = pbids; fa.epids = epids;
  fa.nsamples = nsamples; fa.npt = npt; fa.npv = pv1 - pv0; fa.nkc = nkc; fa.ldt0 = ldt0; fa.npb = npb;
  fa.ng = ng; fa.ldflux = ldflux; fa.dg = dg; fa.flux = flux;
  const int n = pv1 - pv0;
  dim3 fg((npt + 255) / 256, n < 65535 ? n : 65535, (n + 65534) / 65535);
  flux_f64_kernel<<<fg, 256, 0, as_stream(stream)>>>(fa);
  return check_launch("rr_flux_f64");
}

int rr_flux_f64_culled_range(const double* times, const double* tiles64, int npt, const double* k, int nkc,
                             const double* t0, int ldt0, const double* p, int npv, int nlc, int npb,
                             const int32_t* lcids, const int32_t* pbids, const int32_t* epids,
                             const int32_t* nsamples, const double* exptimes, const double* istar, int ng,
                             double dg, const void* workspace, int pv0, int pv1, double* flux, int ldflux,
                             void* stream) {
  if (nkc > 1 && nkc != npb) return RR_ERR_SHAPE;
  if (npt < 0 || npv < 0 || nlc < 1 || npb < 1 || ng < 2 || nkc < 1 || ldflux < npt) return RR_ERR_ARG;
  if (pv0 < 0 || pv1 > npv || pv0 > pv1) return RR_ERR_ARG;
  if (pv1 == pv0 || npt == 0) return RR_OK;
  if (!tiles64) return RR_ERR_ARG;
  Carve cv(const_cast<void*>(workspace));
  double* orb = cv.take<double>((size_t)npv * ORB64);
  double* ldm = cv.take<double>((size_t)npv * npb * ng);
  FluxF64Args fa{};
  fa.times = times; fa.k = k + (size_t)pv0 * nkc; fa.t0 = t0 + (size_t)pv0 * ldt0; fa.p = p + pv0;
  fa.exptimes = exptimes; fa.istar = istar + (size_t)pv0 * npb;
  fa.ldm = ldm + (size_t)pv0 * npb * ng; fa.orb64 = orb + (size_t)pv0 * ORB64;
  fa.lcids = lcids; fa.pbids = pbids; fa.epids = epids;
  fa.nsamples = nsamples; fa.npt = npt; fa.npv = pv1 - pv0; fa.nkc = nkc; fa.ldt0 = ldt0; fa.npb = npb;
  fa.ng = ng; fa.ldflux = ldflux; fa.dg = dg; fa.flux = flux;
  const int n = pv1 - pv0;
  const int ntiles = (npt + TIME_TILE - 1) / TIME_TILE;
  const int tiles_per_block = F64_WARPS * 32;
  dim3 fg((ntiles + tiles_per_block - 1) / tiles_per_block, n < 65535 ? n : 65535, (n + 65534) / 65535);
  flux_f64_culled_kernel<<<fg, F64_WARPS * 32, 0, as_stream(stream)>>>(fa, tiles64);
  return check_launch("rr_flux_f64_culled");
}

int rr_flux_f64(const double* times, int npt, const double* k, int nkc, const double* t0, int ldt0,
                const double* p, int npv, int nlc, int npb, const int32_t* lcids, const int32_t* pbids,
                const int32_t* epids, const int32_t* nsamples, const double* exptimes,
                const double* istar, int ng, double dg, const void* workspace, double* flux, int ldflux,
                void* stream) {
  return rr_flux_f64_range(times, npt, k, nkc, t0, ldt0, p, npv, nlc, npb, lcids, pbids, epids, nsamples, exptimes,
                           istar, ng, dg, workspace, 0, npv, flux, ldflux, stream);
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
                      workspace, workspace_bytes, stream, 0, nullptr, 0, nullptr, 0);
  if (st) return st;
  return rr_flux_f64(times, npt, k, nkc, t0, ldt0, p, npv, nlc, npb, lcids, pbids, epids, nsamples, exptimes,
                     istar, ng, dg, workspace, flux, ldflux, stream);
}

int rr_prepare_split(double t_ref, double t_absmax, const double* k, int nkc, const double* t0, int ldt0,
                     int nep, const double* p, const double* a, const double* inc, const double* e,
                     const double* w, int npv, int nlc, int npb, const int32_t* pbids, const int32_t* epids,
                     const int32_t* nsamples, const double* exptimes, const float* ldp, const float* istar,
                     const float* weights, int nk, int ng, int nz, double dk, double kmin, double kmax,
                     const double* z_edges, void* workspace, size_t workspace_bytes, void* stream, int law,
                     const double* ldc, int npar, const float* basis, int nb) {
  if (nkc > 1 && nkc != npb) return RR_ERR_SHAPE;
  if (npv < 0 || nlc < 1 || npb < 1 || nk < 2 || ng < 2 || nz < 1 || nz > MAX_NZ || nkc < 1 || nep < 1 ||
      nep > ldt0)
    return RR_ERR_ARG;
  if (npv == 0) return RR_OK;
  if (workspace_bytes < rr_full_split_workspace_bytes(npv, npb, nlc, nep, ng)) return RR_ERR_WORKSPACE;
  cudaStream_t s = as_stream(stream);
  SplitTables t = carve_split(workspace, npv, npb, nlc, ng);
  if (basis && nb > 0 && nb <= MAX_BASIS && ldc) {
    ldm_basis_kernel<float><<<npv, 128, sizeof(float) * npb * nb, s>>>(
        law, ldc, npar, npb, k, nkc, basis, nb, nk, ng, dk, kmin, kmax, ldp, nz, z_edges, t.ldm);
  } else {
    ldm_kernel<float><<<ldm_grid(npv, npb, 0), 128, ldm_smem_bytes<float>(ng, nz), s>>>(
        ldp, npb, nz, k, nkc, weights, nk, ng, dk, kmin, kmax, z_edges, 0, nullptr, t.ldm);
  }
  OrbitArgs oa{};
  oa.k = k; oa.t0 = t0; oa.p = p; oa.a = a; oa.inc = inc; oa.e = e; oa.w = w; oa.exptimes = exptimes;
  oa.pbids = pbids; oa.epids = epids; oa.nsamples = nsamples;
  oa.nkc = nkc; oa.ldt0 = ldt0; oa.nep = nep; oa.npv = npv; oa.nlc = nlc; oa.npb = npb; oa.nz = nz;
  oa.ldp = ldp; oa.ldp_is_f32 = 1; oa.orb32 = t.orb; oa.lc32 = t.lc;
  oa.istar32 = istar; oa.t_ref = t_ref; oa.t_absmax = t_absmax;
  orbit_kernel<true><<<(npv + 31) / 32, 32, 0, s>>>(oa);
  return check_launch("rr_prepare_split");
}

int rr_prepare_split_ld(double t_ref, double t_absmax, const double* k, int nkc, const double* t0, int ldt0,
                        int nep, const double* p, const double* a, const double* inc, const double* e,
                        const double* w, int npv, int nlc, int npb, const int32_t* pbids, const int32_t* epids,
                        const int32_t* nsamples, const double* exptimes, int law, const double* ldc, int npar,
                        const double* mu, int nz, const float* basis, int nb, const float* weights, int nk, int ng,
                        double dk, double kmin, double kmax, const double* z_edges, float* ldp, float* istar,
                        void* workspace, size_t workspace_bytes, void* stream) {
  const bool analytic = law == LD_UNIFORM || law == LD_LINEAR || law == LD_QUADRATIC || law == LD_QUADRATIC_TRI;
  const bool fused = analytic && basis && ldc && mu && nb > 0 && nb <= MAX_BASIS && nb == basis_count(law, npar) &&
                     npar >= 0 && npar <= ORB_MAX_LDPAR && npb * npar <= PRO_MAX_COEF && npb * nb <= PRO_MAX_COEF;
  if (!fused) {
    int st = rr_ld_tables_f32(law, ldc, npv, npb, npar, mu, nz, ldp, istar, stream);
    if (st) return st;
    return rr_prepare_split(t_ref, t_absmax, k, nkc, t0, ldt0, nep, p, a, inc, e, w, npv, nlc, npb, pbids, epids,
                            nsamples, exptimes, ldp, istar, weights, nk, ng, nz, dk, kmin, kmax, z_edges, workspace,
                            workspace_bytes, stream, law, ldc, npar, basis, nb);
  }
  if (nkc > 1 && nkc != npb) return RR_ERR_SHAPE;
  if (npv < 0 || nlc < 1 || npb < 1 || nk < 2 || ng < 2 || nz < 1 || nz > MAX_NZ || nkc < 1 || nep < 1 ||
      nep > ldt0 || !ldp || !istar)
    return RR_ERR_ARG;
  if (npv == 0) return RR_OK;
  if (workspace_bytes < rr_full_split_workspace_bytes(npv, npb, nlc, nep, ng)) return RR_ERR_WORKSPACE;
  SplitTables t = carve_split(workspace, npv, npb, nlc, ng);
  ProArgs P{};
  OrbitArgs& oa = P.orb;
  oa.k = k; oa.t0 = t0; oa.p = p; oa.a = a; oa.inc = inc; oa.e = e; oa.w = w; oa.exptimes = exptimes;
  oa.pbids = pbids; oa.epids = epids; oa.nsamples = nsamples;
  oa.nkc = nkc; oa.ldt0 = ldt0; oa.nep = nep; oa.npv = npv; oa.nlc = nlc; oa.npb = npb; oa.nz = nz;
  oa.ldp = nullptr; oa.ldp_is_f32 = 1; oa.orb32 = t.orb; oa.lc32 = t.lc;
  oa.istar32 = nullptr; oa.t_ref = t_ref; oa.t_absmax = t_absmax;
  oa.ld_direct = 1; oa.law = law; oa.npar = npar; oa.ldc = ldc;
  P.npv = npv; P.npb = npb; P.npar = npar; P.nz = nz; P.nb = nb; P.nk = nk; P.ng = ng; P.law = law;
  P.kw_stride = nkc; P.ldc = ldc; P.mu = mu; P.kw = k; P.ze = z_edges;
  P.kmin = kmin; P.kmax = kmax; P.dk = dk; P.inv_dk = 1.0 / dk;
  P.B = basis; P.ldp = ldp; P.istar = istar; P.ldm = t.ldm;
  oa.mu = mu;
  cudaStream_t s = as_stream(stream);
  const int norb = (npv + 31) / 32;
  const int nld = (npv + PRO_WARPS - 1) / PRO_WARPS;
  switch (law) {
    case LD_UNIFORM: prologue_split_kernel<LD_UNIFORM><<<norb + nld, PRO_THREADS, 0, s>>>(P, norb); break;
    case LD_LINEAR: prologue_split_kernel<LD_LINEAR><<<norb + nld, PRO_THREADS, 0, s>>>(P, norb); break;
    case LD_QUADRATIC: prologue_split_kernel<LD_QUADRATIC><<<norb + nld, PRO_THREADS, 0, s>>>(P, norb); break;
    default: prologue_split_kernel<LD_QUADRATIC_TRI><<<norb + nld, PRO_THREADS, 0, s>>>(P, norb); break;
  }
  return check_launch("rr_prepare_split_ld");
}

int rr_flux_split(const float* times_ff, int npt, const int32_t* lcids, int npv, int nlc, int npb, int ng,
                  double dg, const void* workspace, float* flux, int ldflux, void* stream) {
  return rr_flux_split_range(times_ff, npt, lcids, npv, nlc, npb, ng, dg, workspace, 0, npv, flux, ldflux, stream);
}

static int flux_split_args(int npt, int npv, int nlc, int npb, int ng, int pv0, int pv1, int ldflux) {
  if (npt < 0 || npv < 0 || nlc < 1 || npb < 1 || ng < 2 || ldflux < npt) return RR_ERR_ARG;
  if (pv0 < 0 || pv1 > npv || pv0 > pv1) return RR_ERR_ARG;
  return RR_OK;
}

static int flux_split_launch(const float* times_ff, int npt, const int32_t* lcids, int npv, int nlc, int npb,
                             int ng, double dg, const void* workspace, int pv0, int pv1, void* flux, int ldflux,
                             void* stream, int transits_only, bool out_f64) {
  const int st = flux_split_args(npt, npv, nlc, npb, ng, pv0, pv1, ldflux);
  if (st != RR_OK) return st;
  if (pv1 == pv0 || npt == 0) return RR_OK;
  SplitTables t = carve_split(const_cast<void*>(workspace), npv, npb, nlc, ng);
  FluxSplitArgs fa{};
  fa.times_ff = reinterpret_cast<const float2*>(times_ff);
  fa.lcids = lcids;
  // the range's records: the kernel indexes pv from 0 within the range
  fa.orb32 = t.orb + (size_t)pv0 * ORB32;
  fa.lc32 = t.lc + (size_t)pv0 * nlc * LC32;
  fa.ldm = t.ldm + (size_t)pv0 * npb * ng;
  npv = pv1 - pv0;
  fa.npt = npt; fa.npv = npv; fa.npb = npb; fa.nlc = nlc; fa.ng = ng; fa.ldflux = ldflux;
  fa.inv_dg = (float)(1.0 / dg); fa.flux = flux; fa.transits_only = transits_only;
  // tile ranges of FLUX_CHUNK tiles, shorter when the launch would otherwise
  // have fewer than about four blocks per resident warp slot (SMs x 32)
  const int ntiles = (npt + WARP_TILE - 1) / WARP_TILE;
  long long chunk = (long long)ntiles * npv / (4LL * sm_count() * 32);
  chunk = chunk < 1 ? 1 : (chunk > FLUX_CHUNK ? FLUX_CHUNK : chunk);
  const int bx = (int)((ntiles + chunk - 1) / chunk);
  dim3 fg((unsigned)bx, npv < 65535 ? npv : 65535, (npv + 65534) / 65535);
  const bool lc_smem = nlc <= LC_SMEM;
  const size_t smem = sizeof(float) * (ORB32 + (lc_smem ? (size_t)nlc * LC32 : 0));
  cudaStream_t s = as_stream(stream);
  if (out_f64) {
    if (lc_smem)
      flux_split_kernel<true, double><<<fg, FLUX_NW * 32, smem, s>>>(fa, (int)chunk);
    else
      flux_split_kernel<false, double><<<fg, FLUX_NW * 32, smem, s>>>(fa, (int)chunk);
  } else {
    if (lc_smem)
      flux_split_kernel<true, float><<<fg, FLUX_NW * 32, smem, s>>>(fa, (int)chunk);
    else
      flux_split_kernel<false, float><<<fg, FLUX_NW * 32, smem, s>>>(fa, (int)chunk);
  }
  return check_launch("rr_flux_split");
}

// The device address of output rows given as device memory or page-locked
// host memory; NULL for anything else (pageable host memory).
static void* device_rows(void* flux, int* status) {
  *status = RR_OK;
  if (!flux) {
    *status = RR_ERR_ARG;
    return nullptr;
  }
  cudaPointerAttributes at{};
  const cudaError_t e = cudaPointerGetAttributes(&at, flux);
  if (e != cudaSuccess) {
    set_cuda_error(e, "rr_flux_split_transits (pointer)");
    *status = RR_ERR_CUDA;
    return nullptr;
  }
  void* dst = nullptr;
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged)
    dst = flux;
  else if (at.type == cudaMemoryTypeHost)
    dst = at.devicePointer;
  if (!dst) *status = RR_ERR_ARG;   // pageable host memory: not reachable by the kernel here
  return dst;
}

int rr_flux_split_range(const float* times_ff, int npt, const int32_t* lcids, int npv, int nlc, int npb, int ng,
                        double dg, const void* workspace, int pv0, int pv1, float* flux, int ldflux,
                        void* stream) {
  return flux_split_launch(times_ff, npt, lcids, npv, nlc, npb, ng, dg, workspace, pv0, pv1, flux, ldflux, stream,
                           0, false);
}

int rr_flux_split_range_f64(const float* times_ff, int npt, const int32_t* lcids, int npv, int nlc, int npb,
                            int ng, double dg, const void* workspace, int pv0, int pv1, double* flux, int ldflux,
                            void* stream) {
  return flux_split_launch(times_ff, npt, lcids, npv, nlc, npb, ng, dg, workspace, pv0, pv1, flux, ldflux, stream,
                           0, true);
}

int rr_flux_split_transits(const float* times_ff, int npt, const int32_t* lcids, int npv, int nlc, int npb, int ng,
                           double dg, const void* workspace, int pv0, int pv1, float* flux, int ldflux,
                           void* stream) {
  int st = flux_split_args(npt, npv, nlc, npb, ng, pv0, pv1, ldflux);
  if (st != RR_OK || pv1 == pv0 || npt == 0) return st;
  void* dst = device_rows(flux, &st);
  if (!dst) return st;
  return flux_split_launch(times_ff, npt, lcids, npv, nlc, npb, ng, dg, workspace, pv0, pv1, dst, ldflux, stream,
                           1, false);
}

int rr_flux_split_transits_f64(const float* times_ff, int npt, const int32_t* lcids, int npv, int nlc, int npb,
                               int ng, double dg, const void* workspace, int pv0, int pv1, double* flux,
                               int ldflux, void* stream) {
  int st = flux_split_args(npt, npv, nlc, npb, ng, pv0, pv1, ldflux);
  if (st != RR_OK || pv1 == pv0 || npt == 0) return st;
  void* dst = device_rows(flux, &st);
  if (!dst) return st;
  return flux_split_launch(times_ff, npt, lcids, npv, nlc, npb, ng, dg, workspace, pv0, pv1, dst, ldflux, stream,
                           1, true);
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
  st = rr_prepare_split(t_ref, t_absmax, k, nkc, t0, ldt0, nep, p, a, inc, e, w, npv, nlc, npb, pbids, epids,
                        nsamples, exptimes, ldp, istar, weights, nk, ng, nz, dk, kmin, kmax, z_edges, workspace,
                        workspace_bytes, stream, 0, nullptr, 0, nullptr, 0);
  if (st) return st;
  return rr_flux_split(times_ff, npt, lcids, npv, nlc, npb, ng, dg, workspace, flux, ldflux, stream);
}

void rr_full_split_tables(void* workspace, int npv, int npb, int nlc, int nep, int ng, const float** orb32,
                          const float** lc32, const float** ldm) {
  (void)nep;
  SplitTables t = carve_split(workspace, npv, npb, nlc, ng);
  if (orb32) *orb32 = t.orb;
  if (lc32) *lc32 = t.lc;
  if (ldm) *ldm = t.ldm;
}

void rr_serve_struct_sizes(int* request_size, int* item_size) {
  if (request_size) *request_size = (int)sizeof(rr_serve_request);
  if (item_size) *item_size = (int)sizeof(rr_serve_item);
}

int rr_serve_flux_split(const rr_serve_request* reqs, const rr_serve_item* items, const int* nitems, int* counter,
                        int nblocks, void* stream) {
  if (!reqs || !items || !nitems || !counter || nblocks < 1) return RR_ERR_ARG;
  serve_split_kernel<<<nblocks, SPLIT_WARPS * 32, 0, as_stream(stream)>>>(reqs, items, nitems, counter);
  return check_launch("rr_serve_flux_split");
}

int rr_basis_count(int law, int npar) {
  if (law < 0 || law >= LD_NLAWS) return 0;
  return basis_count(law, npar);
}

int rr_basis_tables(int law, int npar, const double* mu, int nz, const double* W64, int nk, int ng, double* B64,
                    float* B32, void* stream) {
  const int nb = rr_basis_count(law, npar);
  if (nb <= 0 || nb > MAX_BASIS || nk < 2 || ng < 2 || nz < 1 || !mu || !W64 || !B64) return RR_ERR_ARG;
  basis_tables_kernel<<<(nk * ng + 127) / 128, 128, 0, as_stream(stream)>>>(law, nb, mu, nz, W64, nk, ng, B64, B32);
  return check_launch("rr_basis_tables");
}

}  // extern "C"
