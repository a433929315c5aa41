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

__global__ void time_split_kernel(const double* __restrict__ times, int npt, double t_ref,
                                  float2* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npt) return;
  double dt = times[i] - t_ref;
  float hi = __double2float_rn(dt);
  float lo = __double2float_rn(dt - (double)hi);
  out[i] = make_float2(hi, lo);
}

constexpr int MAX_LDPAR = 16;
constexpr int NTRAP = 200;

// evaluate_ld + evaluate_ldi (ldmodels.py:143-174) or the 200-point trapezoid
// of rrmodel.py:222-227, one thread per (pv, pb).
template <typename R>
__global__ void ld_tables_kernel(int law, const double* __restrict__ ldc, int npvpb, int npar,
                                 const double* __restrict__ mu, int nz, R* __restrict__ ldp,
                                 R* __restrict__ istar) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= npvpb) return;
  R pv[MAX_LDPAR];
  for (int i = 0; i < npar; ++i) pv[i] = (R)ldc[(size_t)j * npar + i];
  for (int i = 0; i < nz; ++i) ldp[(size_t)j * nz + i] = ld_value<R>(law, (R)mu[i], pv, npar);
  R is;
  if (!ld_integral<R>(law, pv, is)) {
    // 2*pi*trapezoid(z*I(mu(z)), z), mu = linspace(1, 0, 200), z = sqrt(1 - mu^2)
    R s = R(0), z0 = R(0), y0 = R(0);
    for (int i = 0; i < NTRAP; ++i) {
      // (n-1-i)/(n-1): exactly 1 and 0 at the ends (a select of the end value
      // was not honoured by the nvcc 13.0 -O3 build, leaving mu = -1.5e-17)
      R m = R(NTRAP - 1 - i) / R(NTRAP - 1);
      R z = sqrt(R(1) - m * m);
      R y = z * ld_value<R>(law, m, pv, npar);
      if (i > 0) s += (z - z0) * (y + y0) / R(2);
      z0 = z;
      y0 = y;
    }
    is = R(2.0 * PI) * s;
  }
  istar[j] = is;
}

template <typename R>
static int ld_tables(int law, const double* ldc, int npv, int npb, int npar, const double* mu, int nz,
                     R* ldp, R* istar, void* stream) {
  if (law < 0 || law >= LD_NLAWS) return RR_ERR_LAW;
  if (npv < 0 || npb < 1 || npar < 0 || npar > MAX_LDPAR || nz < 1) return RR_ERR_ARG;
  int n = npv * npb;
  if (n == 0) return RR_OK;
  ld_tables_kernel<R><<<(n + 127) / 128, 128, 0, as_stream(stream)>>>(law, ldc, n, npar, mu, nz, ldp, istar);
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

int rr_time_split(const double* times, int npt, double t_ref, float* times_ff, void* stream) {
  if (npt < 0 || (npt > 0 && (!times || !times_ff))) return RR_ERR_ARG;
  if (npt == 0) return RR_OK;
  time_split_kernel<<<(npt + 255) / 256, 256, 0, as_stream(stream)>>>(
      times, npt, t_ref, reinterpret_cast<float2*>(times_ff));
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
