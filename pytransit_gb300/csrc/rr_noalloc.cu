// Split-precision RoadRunner evaluation for callers that cannot allocate GPU
// memory.  Examples are plugin hosts that own the device and hand a plugin
// only its input and output buffers, memory-pool based runtimes that forbid
// raw cudaMalloc, and latency-bound loops where a cudaMalloc (which may
// synchronise the device) is not acceptable.  Instead of a caller-provided
// workspace, the per-parameter-vector tables live in a fixed, file-scope
// device array that every GPU loading this library keeps until process exit.
#include <cuda.h>   // the driver's context types, for the context check below

#include <mutex>

#include "rr_internal.h"

namespace rr {

// Fixed scratch for rr_full_split_noalloc: 32 MiB, enough for e.g. 16k
// parameter vectors with 4 passbands and 4 light curves.
constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(32) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
static void* g_scratch_addr[MAX_DEVICES] = {};
static unsigned long long g_scratch_ctx[MAX_DEVICES] = {};
static std::mutex g_scratch_mutex;

// The id of the current CUDA context (cuCtxGetId, reached through the runtime's
// driver entry points so that the library links the runtime only), or 0 if it
// cannot be had.  A device reset, or a primary context released and made
// again, gives the device a new context id and the module a new address.
static unsigned long long current_context_id() {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", reinterpret_cast<void**>(&get_current), 12000,
                                         cudaEnableDefault, &q1) != cudaSuccess || q1 != cudaDriverEntryPointSuccess)
      get_current = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", reinterpret_cast<void**>(&get_id), 12000, cudaEnableDefault,
                                         &q2) != cudaSuccess || q2 != cudaDriverEntryPointSuccess)
      get_id = nullptr;
    looked_up = true;
  }
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of the scratch array on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// with the device current, once per device and context, and cached; a call
// in a context other than the cached one (after a device reset, say) looks it
// up again.
static int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_cuda_error(e, "rr_full_split_noalloc: cudaGetDevice");
    return RR_ERR_CUDA;
  }
  if (dev < 0 || dev >= MAX_DEVICES) {
    set_error_text("rr_full_split_noalloc", "device index beyond the 64 devices the scratch cache covers");
    return RR_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  const unsigned long long ctx = current_context_id();
  if (g_scratch_addr[dev] == nullptr || ctx == 0 || ctx != g_scratch_ctx[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      set_cuda_error(e, "rr_full_split_noalloc: cudaGetSymbolAddress");
      return RR_ERR_CUDA;
    }
    g_scratch_addr[dev] = p;
    g_scratch_ctx[dev] = current_context_id();   // the lookup has made the context current if it was not
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
