// Split-precision RoadRunner evaluation for callers that cannot allocate GPU
// memory.  Examples are plugin hosts that own the device and hand a plugin
// only its input and output buffers, memory-pool based runtimes that forbid
// raw cudaMalloc, and latency-bound loops where a cudaMalloc (which may
// synchronise the device) is not acceptable.  Instead of a caller-provided
// workspace, the per-parameter-vector tables live in a fixed, file-scope
// device array that every GPU loading this library keeps until process exit.
#include <mutex>

#include "rr_internal.h"

namespace rr {

// Fixed scratch for rr_full_split_noalloc: 32 MiB, enough for e.g. 16k
// parameter vectors with 4 passbands and 4 light curves.
constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
static void* g_scratch_addr[MAX_DEVICES] = {};
static std::mutex g_scratch_mutex;

// Device address of the scratch array on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// once per device (with that device current) and cached.
static int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_cuda_error(e, "rr_full_split_noalloc: cudaGetDevice");
    return RR_ERR_CUDA;
  }
  if (dev < 0 || dev >= MAX_DEVICES) return RR_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_addr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_cuda_error(e, "rr_full_split_noalloc: cudaGetSymbolAddress");
      return RR_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return RR_OK;
}

}  // namespace rr

using namespace rr;

extern "C" {

size_t rr_full_split_noalloc_max_bytes(void) { return NOALLOC_SCRATCH_BYTES; }

int rr_full_split_noalloc(const float* times_ff, double t_ref, double t_absmax, int npt, const double* k,
                          int nkc, const double* t0, int ldt0, int nep, const double* p, const double* a,
                          const double* inc, const double* e, const double* w, int npv, int nlc, int npb,
                          const int32_t* lcids, const int32_t* pbids, const int32_t* epids,
                          const int32_t* nsamples, const double* exptimes, const float* ldp,
                          const float* istar, const float* weights, int nk, int ng, int nz, double dk,
                          double kmin, double kmax, double dg, const double* z_edges, float* flux,
                          int ldflux, void* stream) {
  if (npv < 0 || npb < 1 || nlc < 1 || nep < 1 || ng < 2) return RR_ERR_ARG;
  const size_t need = rr_full_split_workspace_bytes(npv, npb, nlc, nep, ng);
  if (need > NOALLOC_SCRATCH_BYTES) return RR_ERR_WORKSPACE;
  void* scratch = nullptr;
  int st = scratch_address(&scratch);
  if (st) return st;
  // Every table in the scratch is written by the prologue before the flux
  // kernel reads it, so nothing has to be cleared between calls.
  return rr_full_split(times_ff, t_ref, t_absmax, npt, k, nkc, t0, ldt0, nep, p, a, inc, e, w, npv, nlc, npb,
                       lcids, pbids, epids, nsamples, exptimes, ldp, istar, weights, nk, ng, nz, dk, kmin, kmax,
                       dg, z_edges, scratch, NOALLOC_SCRATCH_BYTES, flux, ldflux, stream);
}

}  // extern "C"
