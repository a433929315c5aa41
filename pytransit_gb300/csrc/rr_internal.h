// Host-side helpers shared by the translation units of the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

#include "../../include/pytransit_gb300.h"

namespace rr {

// Records the CUDA error (if any) of the last launch on this host thread.
int check_launch(const char* where);
void set_cuda_error(cudaError_t e, const char* where);
// Records a message of the library's own (not a CUDA error) for rr_last_cuda_error.
void set_error_text(const char* where, const char* what);

// LD-means kernel launchers (rr_full.cu); mode 0: rr_full rule, 1: the
// transmission-spectroscopy rule with kmax_pv, 2: always the 2D table.
void launch_ldm_f32(const float* ldp, int npv, int npb, int nz, const double* kw, int kw_stride, const float* W,
                    int nk, int ng, double dk, double kmin, double kmax, const double* ze, int mode,
                    const double* kmax_pv, float* ldm, cudaStream_t s);
void launch_ldm_f64(const double* ldp, int npv, int npb, int nz, const double* kw, int kw_stride, const double* W,
                    int nk, int ng, double dk, double kmin, double kmax, const double* ze, int mode,
                    const double* kmax_pv, double* ldm, cudaStream_t s);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Multiprocessor count of the current device (queried once per device), for
// launch shapes.
int sm_count();

// Bump allocator over a caller-owned workspace (256-byte aligned pieces).
struct Carve {
  char* base;
  size_t used;
  explicit Carve(void* b) : base(static_cast<char*>(b)), used(0) {}
  template <typename T>
  T* take(size_t n) {
    used = (used + 255) & ~size_t(255);
    T* p = reinterpret_cast<T*>(base ? base + used : nullptr);
    used += n * sizeof(T);
    return p;
  }
};

// Per-parameter-vector record of the plain FP64 path (16 doubles):
// c[0..9] Taylor coefficients, [10] t1, [11] t4 (contact times), [12] valid.
constexpr int ORB64 = 16;
// Per-parameter-vector record of the split path (16 floats):
// c[0..9], [10] p_hi, [11] p_lo, [12] 1/p, [13] fast-test error bound,
// [14] flags (int bits), [15] unused.
constexpr int ORB32 = 16;
// Per-(pv, light curve) record of the split path (16 floats).
constexpr int LC32 = 16;
enum LcField {
  LC_FLO = 0, LC_FHI = 1,     // fast-test box (widened by the error bound)
  LC_D0H = 2, LC_D0L = 3,     // t0[pv, epoch of lc] - t_ref as an FP32 pair
  LC_LO = 4, LC_HI = 5,       // bounding box incl. the 0.003 d + exptime pad
  LC_K = 6, LC_INV1PK = 7,    // radius ratio of the lc's passband, 1/(1+k)
  LC_INVIS = 8,               // 1/istar of the passband (NaN if istar is not finite)
  LC_EXPT = 9, LC_INVNS = 10, // exposure time, 1/nsamples
  LC_NS = 11, LC_PB = 12      // nsamples, passband (int bits)
};
// Points per time tile (one warp, four points per lane).  The FP32-pair time
// array holds 2 * round_up(npt, 2) floats followed by one float4 per tile:
// (min hi, max hi, light curve id or -1 as int bits, 0).
constexpr int TIME_TILE = 128;
__host__ __device__ inline size_t time_meta_offset(int npt) { return 2 * (((size_t)npt + 1) / 2 * 2); }
constexpr int FLAG_VALID = 1;
constexpr int FLAG_WIDE = 2;  // box too close to +-p/2: take the exact path for every point

}  // namespace rr
