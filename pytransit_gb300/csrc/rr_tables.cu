// Model initialisation and data-side kernels: the RoadRunner weight table,
// the FP32-pair time split and the limb-darkening tables, plus the ABI's
// status helpers.
#include <cstdio>
#include <cmath>

#include "rr_device.cuh"
#include "rr_internal.h"

namespace rr {

static thread_local char g_last_error[256] = "no error";

void set_cuda_error(cudaError_t e, const char* where) {
  snprintf(g_last_error, sizeof(g_last_error), "%s: %s", where, cudaGetErrorString(e));
}

void set_error_text(const char* where, const char* what) {
  snprintf(g_last_error, sizeof(g_last_error), "%s: %s", where, what);
}

int sm_count() {
  constexpr int kMaxDev = 64;
  static int cached[kMaxDev] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 152;
  if (dev < kMaxDev && cached[dev] > 0) return cached[dev];
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) n = 152;
  if (dev < kMaxDev) cached[dev] = n;
  return n;
}

int check_launch(const char* where) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_cuda_error(e, where);
    return RR_ERR_CUDA;
  }
  return RR_OK;
}

// numpy.linspace element: i*step + start, the last element exactly stop.
__device__ __forceinline__ double linspace_at(double start, double stop, int num, int i) {
  if (i == num - 1) return stop;
  double step = (stop - start) / (double)(num - 1);
  return (double)i * step + start;
}

// One (k, g) row of calculate_weights_3d, common.py:210-222.
__global__ void weights_3d_kernel(int nk, double kmin, double kmax, const double* __restrict__ ze,
                                  int nz, int ng, double* __restrict__ W64, float* __restrict__ W32) {
  int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= nk * ng) return;
  int ik = row / ng, ig = row % ng;
  double k = linspace_at(kmin, kmax, nk, ik);
  double g = linspace_at(0.0, 1.0 - 1e-7, ng, ig);
  double b = g * (1.0 + k);
  double* out = W64 + (size_t)row * nz;
  double a0 = cci_acos(ze[0], k, b);
  out[0] = a0;
  double s = a0;
  for (int i = 1; i < nz; ++i) {
    double a1 = cci_acos(ze[i], k, b);
    out[i] = a1 - a0;
    a0 = a1;
    s += out[i];
  }
  for (int i = 0; i < nz; ++i) {
    out[i] /= s;
    if (W32) W32[(size_t)row * nz + i] = (float)out[i];
  }
}

// One warp per 128-point tile: the FP32-pair times (hi, lo) of t - t_ref and
// the tile's summary (min and max of hi, its light curve or -1 if mixed),
// which lets the flux kernel skip tiles far from every transit.
__global__ void time_split_kernel(const double* __restrict__ times, const int32_t* __restrict__ lcids, int npt,
                                  double t_ref, float2* __restrict__ out, float4* __restrict__ meta) {
  const int tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int ntiles = (npt + TIME_TILE - 1) / TIME_TILE;
  if (tile >= ntiles) return;  // warp-uniform
  float tmin = INFINITY, tmax = -INFINITY;
  int lc = -2;
  bool same = true;
  for (int q = 0; q < 4; ++q) {
    const int i = tile * TIME_TILE + lane * 4 + q;
    if (i < npt) {
      const double dt = times[i] - t_ref;
      const float hi = __double2float_rn(dt);
      const float lo = __double2float_rn(dt - (double)hi);
      out[i] = make_float2(hi, lo);
      tmin = fminf(tmin, hi);
      tmax = fmaxf(tmax, hi);
      const int l = lcids[i];
      if (lc == -2) lc = l;
      same = same && (l == lc);
    }
  }
  const unsigned FULL = 0xffffffffu;
  for (int o = 16; o > 0; o >>= 1) {
    tmin = fminf(tmin, __shfl_xor_sync(FULL, tmin, o));
    tmax = fmaxf(tmax, __shfl_xor_sync(FULL, tmax, o));
  }
  const int lc0 = __shfl_sync(FULL, lc, 0);
  same = __all_sync(FULL, same && (lc == -2 || lc == lc0));
  if (lane == 0) meta[tile] = make_float4(tmin, tmax, __int_as_float(same ? lc0 : -1), 0.0f);
}

// One warp per 128-point tile: the FP64 summary of the tile for the culled
// FP64 flux kernel, (earliest time, latest time, light curve or -1 when the
// tile holds several, 0).
__global__ void time_tiles_f64_kernel(const double* __restrict__ times, const int32_t* __restrict__ lcids, int npt,
                                      double* __restrict__ tiles) {
  const int tile = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int ntiles = (npt + TIME_TILE - 1) / TIME_TILE;
  if (tile >= ntiles) return;  // warp-uniform
  double tmin = INFINITY, tmax = -INFINITY;
  int lc = -2;
  bool same = true;
  for (int q = 0; q < 4; ++q) {
    const int i = tile * TIME_TILE + lane * 4 + q;
    if (i < npt) {
      const double t = times[i];
      tmin = fmin(tmin, t);
      tmax = fmax(tmax, t);
      const int l = lcids[i];
      if (lc == -2) lc = l;
      same = same && (l == lc);
    }
  }
  const unsigned FULL = 0xffffffffu;
  for (int o = 16; o > 0; o >>= 1) {
    tmin = fmin(tmin, __shfl_xor_sync(FULL, tmin, o));
    tmax = fmax(tmax, __shfl_xor_sync(FULL, tmax, o));
  }
  const int lc0 = __shfl_sync(FULL, lc, 0);
  same = __all_sync(FULL, same && (lc == -2 || lc == lc0));
  if (lane == 0) {
    double* o = tiles + 4 * (size_t)tile;
    o[0] = tmin;
    o[1] = tmax;
    o[2] = (same && lc0 >= 0) ? (double)lc0 : -1.0;
    o[3] = 0.0;
  }
}

constexpr int MAX_LDPAR = 16;
constexpr int NTRAP = 200;

// evaluate_ld + evaluate_ldi (ldmodels.py:143-174) or the 200-point trapezoid
// of rrmodel.py:222-227, one warp per (pv, pb): lanes over the mu grid, and
// over the trapezoid's intervals with a warp sum.
template <typename R>
__global__ void __launch_bounds__(128) ld_tables_kernel(int law, const double* __restrict__ ldc, int npvpb, int npar,
                                                        const double* __restrict__ mu, int nz, R* __restrict__ ldp,
                                                        R* __restrict__ istar) {
  const int j = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= npvpb) return;   // warp-uniform
  R pv[MAX_LDPAR];
  for (int i = 0; i < npar; ++i) pv[i] = (R)ldc[(size_t)j * npar + i];
  for (int i = lane; i < nz; i += 32) ldp[(size_t)j * nz + i] = ld_value<R>(law, (R)mu[i], pv, npar);
  R is;
  if (!ld_integral<R>(law, pv, is)) {
    // 2*pi*trapezoid(z*I(mu(z)), z), mu = linspace(1, 0, 200), z = sqrt(1 - mu^2);
    // lane l takes the intervals i = l, l + 32, ...
    R s = R(0);
    for (int i = lane + 1; i < NTRAP; i += 32) {
      // (n-1-i)/(n-1): exactly 1 and 0 at the ends (a select of the end value
      // was not honoured by the nvcc 13.0 -O3 build, leaving mu = -1.5e-17)
      const R m0 = R(NTRAP - i) / R(NTRAP - 1), m1 = R(NTRAP - 1 - i) / R(NTRAP - 1);
      const R z0 = sqrt(R(1) - m0 * m0), z1 = sqrt(R(1) - m1 * m1);
      const R y0 = z0 * ld_value<R>(law, m0, pv, npar), y1 = z1 * ld_value<R>(law, m1, pv, npar);
      s += (z1 - z0) * (y1 + y0) / R(2);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    is = R(2.0 * PI) * s;
  }
  if (lane == 0) istar[j] = is;
}

template <typename R>
static int ld_tables(int law, const double* ldc, int npv, int npb, int npar, const double* mu, int nz,
                     R* ldp, R* istar, void* stream) {
  if (law < 0 || law >= LD_NLAWS) return RR_ERR_LAW;
  if (npv < 0 || npb < 1 || npar < 0 || npar > MAX_LDPAR || nz < 1) return RR_ERR_ARG;
  const long long n = (long long)npv * npb;
  if (n == 0) return RR_OK;
  ld_tables_kernel<R><<<(unsigned)((n + 3) / 4), 128, 0, as_stream(stream)>>>(law, ldc, (int)n, npar, mu, nz, ldp,
                                                                              istar);
  return check_launch("rr_ld_tables");
}

}  // namespace rr

using namespace rr;

extern "C" {

int rr_abi_version(void) { return 1; }

const char* rr_status_string(int status) {
  switch (status) {
    case RR_OK: return "ok";
    case RR_ERR_SHAPE: return "Radius ratios should be given either as an [npv, 1] or [npv, npb] array.";
    case RR_ERR_ARG: return "invalid argument";
    case RR_ERR_WORKSPACE: return "workspace too small";
    case RR_ERR_CUDA: return "CUDA error";
    case RR_ERR_LAW: return "unknown limb darkening law";
    case RR_ERR_TIMEOUT: return "device wait timed out";
  }
  return "unknown status";
}

const char* rr_last_cuda_error(void) { return g_last_error; }

int rr_weights_3d(int nk, double kmin, double kmax, const double* ze, int nz, int ng, double* W64,
                  float* W32, double* dk, double* dg, void* stream) {
  if (nk < 2 || ng < 2 || nz < 1 || !ze || !W64) return RR_ERR_ARG;
  int rows = nk * ng;
  weights_3d_kernel<<<(rows + 127) / 128, 128, 0, as_stream(stream)>>>(nk, kmin, kmax, ze, nz, ng, W64, W32);
  if (dk) *dk = (kmax - kmin) / nk;
  // dg = gs[1] - gs[0] of gs = linspace(0, 1 - 1e-7, ng)
  if (dg) *dg = (ng == 2) ? (1.0 - 1e-7) : (1.0 - 1e-7) / (double)(ng - 1);
  return check_launch("rr_weights_3d");
}

size_t rr_time_tiles_f64_doubles(int npt) {
  if (npt < 0) return 0;
  return 4 * (((size_t)npt + TIME_TILE - 1) / TIME_TILE);
}

int rr_time_tiles_f64(const double* times, const int32_t* lcids, int npt, double* tiles64, void* stream) {
  if (npt < 0 || (npt > 0 && (!times || !lcids || !tiles64))) return RR_ERR_ARG;
  if (npt == 0) return RR_OK;
  const int ntiles = (npt + TIME_TILE - 1) / TIME_TILE;
  time_tiles_f64_kernel<<<(ntiles * 32 + 255) / 256, 256, 0, as_stream(stream)>>>(times, lcids, npt, tiles64);
  return check_launch("rr_time_tiles_f64");
}

size_t rr_time_split_floats(int npt) {
  if (npt < 0) return 0;
  const size_t ntiles = ((size_t)npt + TIME_TILE - 1) / TIME_TILE;
  return 2 * (((size_t)npt + 1) / 2 * 2) + 4 * ntiles;
}

int rr_time_split(const double* times, const int32_t* lcids, int npt, double t_ref, float* times_ff,
                  void* stream) {
  if (npt < 0 || (npt > 0 && (!times || !lcids || !times_ff))) return RR_ERR_ARG;
  if (npt == 0) return RR_OK;
  const int ntiles = (npt + TIME_TILE - 1) / TIME_TILE;
  float4* meta = reinterpret_cast<float4*>(times_ff + 2 * (((size_t)npt + 1) / 2 * 2));
  time_split_kernel<<<(ntiles * 32 + 255) / 256, 256, 0, as_stream(stream)>>>(
      times, lcids, npt, t_ref, reinterpret_cast<float2*>(times_ff), meta);
  return check_launch("rr_time_split");
}

int rr_ld_tables_f64(int law, const double* ldc, int npv, int npb, int npar, const double* mu, int nz,
                     double* ldp, double* istar, void* stream) {
  return ld_tables<double>(law, ldc, npv, npb, npar, mu, nz, ldp, istar, stream);
}

int rr_ld_tables_f32(int law, const double* ldc, int npv, int npb, int npar, const double* mu, int nz,
                     float* ldp, float* istar, void* stream) {
  return ld_tables<float>(law, ldc, npv, npb, npar, mu, nz, ldp, istar, stream);
}

}  // extern "C"
