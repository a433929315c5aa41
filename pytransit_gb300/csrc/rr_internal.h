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

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

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
constexpr int FLAG_VALID = 1;
constexpr int FLAG_WIDE = 2;  // box too close to +-p/2: take the exact path for every point

}  // namespace rr
