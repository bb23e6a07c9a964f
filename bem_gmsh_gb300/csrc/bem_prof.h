// Kernel-class timing and launch counting inside the library.  Timing uses
// CUDA events recorded on the stream each kernel class runs on; it is off
// unless enabled with BEM_OPT_KERNEL_TIMING.  The launch counter is always on.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <vector>

namespace bem {

enum KClass {
  KC_FAR = 0,        // far-field tile kernel
  KC_NEAR = 1,       // near-singular + on-element + diagonal kernels
  KC_LU_PREP = 2,    // equilibration + FP32 copy
  KC_LU_CRIT = 3,    // diagonal blocks, panels (lookahead stream)
  KC_LU_TRAIL = 4,   // bulk trailing updates (tcgen05)
  KC_TRSV = 5,       // triangular solves
  KC_GEMV = 6,       // FP64 matrix-vector products / residuals
  KC_LU_TOTAL = 7,   // whole factorization
  KC_LU_DIAG = 8,    // diagonal-block factorizations (within KC_LU_CRIT)
  KC_LU_PANELS = 9,  // block row / column panels (within KC_LU_CRIT)
  KC_LU_THIN = 10,   // look-ahead updates of the next block row / column (within KC_LU_CRIT)
  KC_COUNT = 11
};

struct KProf {
  bool on = false;
  struct Rec {
    cudaEvent_t a, b;
    int cls;
  };
  std::vector<Rec> pending;
  std::vector<cudaEvent_t> pool;
  double ms[KC_COUNT] = {0};
  long long n[KC_COUNT] = {0};
  // timeline of the collected records: class, start and end in ms from the
  // start of the first record of each collection
  struct Span {
    int cls;
    double t0, t1;
  };
  std::vector<Span> trace;

  cudaEvent_t ev() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  cudaEvent_t begin(cudaStream_t s) {
    if (!on) return nullptr;
    cudaEvent_t a = ev();
    cudaEventRecord(a, s);
    return a;
  }
  void end(cudaStream_t s, cudaEvent_t a, int cls) {
    if (!on || !a) return;
    cudaEvent_t b = ev();
    cudaEventRecord(b, s);
    pending.push_back({a, b, cls});
  }
  // call after the streams were synchronized
  void collect() {
    for (auto& r : pending) {
      float v = 0.f;
      if (cudaEventElapsedTime(&v, r.a, r.b) == cudaSuccess) {
        ms[r.cls] += v;
        n[r.cls] += 1;
        float s0 = 0.f;
        if (trace.size() < (1u << 16) && cudaEventElapsedTime(&s0, pending[0].a, r.a) == cudaSuccess)
          trace.push_back({r.cls, (double)s0, (double)s0 + v});
      }
      pool.push_back(r.a);
      pool.push_back(r.b);
    }
    pending.clear();
  }
  void release() {
    collect();
    for (auto e : pool) cudaEventDestroy(e);
    pool.clear();
  }
};

// process-wide count of kernel launches made by the library
extern std::atomic<long long> g_launches;
// launches issued by this thread (a graph capture measures its own)
extern thread_local long long tl_launches;
inline void count_launches(long long k) {
  g_launches.fetch_add(k, std::memory_order_relaxed);
  tl_launches += k;
}

// profiler of the context whose C-ABI call is running on this thread
extern thread_local KProf* tl_prof;

// times the work enqueued on `s` during its lifetime as class `cls`
struct KScope {
  cudaStream_t s;
  cudaEvent_t a;
  int cls;
  KScope(cudaStream_t s_, int c) : s(s_), a(nullptr), cls(c) {
    if (tl_prof) a = tl_prof->begin(s);
  }
  ~KScope() {
    if (tl_prof) tl_prof->end(s, a, cls);
  }
};

}  // namespace bem
