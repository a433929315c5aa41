// Host-side fill of output rows on the library's own threads
// (rr_host_fill_f32).  With rr_flux_split_transits it lets the host set a
// chunk of flux rows to 1 while the GPU writes only the tiles of the previous
// chunk that reach a transit: culled tiles then never cross the host link.
//
// A small pool of worker threads is started on first use and kept for the
// life of the process (never joined: its threads are detached, so process
// exit does not wait on them).  A call splits [0, n) into equal 64-byte
// aligned slices, one per thread, the calling thread taking the last; it
// returns when every slice is written.  Calls are serialised by a mutex.  A
// process forked after the pool started gets a new pool on its next call.
#include <unistd.h>

#include <algorithm>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <mutex>
#include <thread>
#include <vector>

#include "rr_internal.h"

namespace {

struct FillPool {
  std::mutex call;                 // one fill at a time
  std::mutex m;
  std::condition_variable go, done;
  unsigned long long generation = 0;
  int workers = 0;
  int remaining = 0;
  void* dst = nullptr;
  size_t n = 0;
  double value = 0.0;
  bool f64 = false;
  int parts = 1;
  pid_t owner = 0;

  template <typename T>
  static void fill_slice_t(T* dst, size_t n, T value, int parts, int part) {
    // slices are whole 64-byte blocks except the last
    constexpr size_t B = 64 / sizeof(T);
    const size_t blocks = (n + B - 1) / B;
    const size_t per = (blocks + parts - 1) / parts;
    const size_t b0 = std::min(blocks, per * (size_t)part), b1 = std::min(blocks, b0 + per);
    const size_t i0 = b0 * B, i1 = std::min(n, b1 * B);
    T* p = dst + i0;
    for (size_t i = i0; i < i1; ++i) *p++ = value;
  }

  static void fill_slice(void* dst, size_t n, double value, bool f64, int parts, int part) {
    if (f64)
      fill_slice_t<double>(static_cast<double*>(dst), n, value, parts, part);
    else
      fill_slice_t<float>(static_cast<float*>(dst), n, (float)value, parts, part);
  }

  void worker(int id, unsigned long long seen) {
    for (;;) {
      void* d;
      size_t nn;
      double v;
      bool dbl;
      int np;
      {
        std::unique_lock<std::mutex> lk(m);
        go.wait(lk, [&] { return generation != seen; });
        seen = generation;
        d = dst; nn = n; v = value; dbl = f64; np = parts;
      }
      if (id < np - 1) fill_slice(d, nn, v, dbl, np, id);
      std::lock_guard<std::mutex> lk(m);
      if (--remaining == 0) done.notify_one();
    }
  }

  void ensure(int nworkers) {
    // a new worker starts from the current generation, so that it takes no
    // earlier call's task for its own; a thread that cannot be started (a
    // process limit) leaves the pool as large as it got
    std::lock_guard<std::mutex> lk(m);
    while (workers < nworkers) {
      try {
        std::thread(&FillPool::worker, this, workers, generation).detach();
      } catch (...) {
        return;
      }
      ++workers;
    }
  }

  void run(void* d, size_t nn, double v, bool dbl, int nthreads) {
    std::lock_guard<std::mutex> serial(call);
    int np = std::max(1, nthreads);
    if (np > 1) ensure(np - 1);
    np = std::min(np, workers + 1);   // the slices go to the threads there are
    if (np == 1) {
      fill_slice(d, nn, v, dbl, 1, 0);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(m);
      dst = d; n = nn; value = v; f64 = dbl; parts = np;
      remaining = workers;   // every worker wakes and reports, busy or not
      ++generation;
    }
    go.notify_all();
    fill_slice(d, nn, v, dbl, np, np - 1);
    std::unique_lock<std::mutex> lk(m);
    done.wait(lk, [&] { return remaining == 0; });
  }
};

FillPool* g_pool = nullptr;
std::mutex g_pool_mu;

FillPool* pool() {
  std::lock_guard<std::mutex> lk(g_pool_mu);
  const pid_t me = getpid();
  if (!g_pool || g_pool->owner != me) {
    // a forked child inherits the parent's pool without its threads: start
    // afresh (the parent's pool object is left as it is)
    g_pool = new FillPool();
    g_pool->owner = me;
  }
  return g_pool;
}

}  // namespace

static int host_fill(void* dst, size_t n, double value, bool f64, int nthreads) {
  if (n == 0) return RR_OK;
  if (!dst) return RR_ERR_ARG;
  if (nthreads > 256) nthreads = 256;
  // small fills are not worth a wake-up of the pool
  if (n < ((size_t)1 << 16)) nthreads = 1;
  pool()->run(dst, n, value, f64, nthreads);
  return RR_OK;
}

extern "C" int rr_host_fill_f32(float* dst, size_t n, float value, int nthreads) {
  return host_fill(dst, n, value, false, nthreads);
}

extern "C" int rr_host_fill_f64(double* dst, size_t n, double value, int nthreads) {
  return host_fill(dst, n, value, true, nthreads);
}
