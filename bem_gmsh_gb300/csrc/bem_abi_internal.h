// Context object and helpers shared by the C-ABI translation units.
#pragma once
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/bem_gb300.h"
#include "bem_kernels.h"
#include "bem_prof.h"

struct bem_ctx {
  enum Slot {
    SLOT_GEOM, SLOT_ROWS, SLOT_NODES, SLOT_ELEMS, SLOT_ROWSUM, SLOT_GDIAG, SLOT_COUNTERS,
    SLOT_PAIRS, SLOT_BC, SLOT_BV, SLOT_OUT0, SLOT_OUT1, SLOT_OUT2, SLOT_OUT3,
    SLOT_LU0, SLOT_LU1, SLOT_LU2, SLOT_LU3, SLOT_LU4, SLOT_LU5, SLOT_LU6, SLOT_LU7,
    SLOT_TC0, SLOT_TC1, SLOT_TC2, SLOT_TC3, SLOT_TC4, SLOT_TC5, SLOT_TEST0, SLOT_TEST1,
    SLOT_NODES_DF, SLOT_LOGTAB, SLOT_ADJ0, SLOT_ADJ1, SLOT_LU8,
    NSLOT
  };
  struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
  };
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string last_error;
  Buf slots[NSLOT];
  int pair_cap_hint = 0;
  int opt_tcgen05 = 2;  // BEM_OPT_TCGEN05: trailing updates on tcgen05 (2: persistent kernel)
  int opt_tc_reserve = 0;  // BEM_OPT_TC_RESERVE: SMs the persistent kernel leaves free
  int opt_far_df = 1;   // BEM_OPT_FAR_DF
  int opt_graphs = 1;   // BEM_OPT_GRAPHS
  int opt_pivot_fallback = 1;      // BEM_OPT_PIVOT_FALLBACK
  int opt_wait_limit = 1 << 20;    // BEM_OPT_WAIT_LIMIT
  int opt_inject = 0;              // BEM_OPT_INJECT
  int opt_nearfield = 0;           // BEM_OPT_NEARFIELD
  int opt_singular = 0;            // BEM_OPT_SINGULAR
  int opt_sweep_ctas = 4;          // BEM_OPT_SWEEP_CTAS: CTAs per block row of the triangular sweeps
  // why the last mixed solve did not converge (MIXED_*)
  enum { MIXED_OK = 0, MIXED_PIVOT = 1, MIXED_STAGNATION = 2, MIXED_CAP = 3 };
  int mixed_fail = MIXED_OK;
  // captured factorization of the mixed solve, replayed while the buffers and
  // sizes in its key are unchanged (captured on the second call with a key)
  cudaGraphExec_t lu_graph = nullptr;
  std::vector<const void*> lu_graph_key;
  long long lu_graph_launches = 0;
  int lu_graph_calls = 0;
  void* cusolver_handle = nullptr;  // FP64 comparison path (created on first use)
  std::vector<bem_ctx*> workers;    // sub-contexts of batched calls (own streams)
  // side stream and events of the assembly (created on first use)
  cudaStream_t asm_stream = nullptr, asm_stream2 = nullptr;
  cudaEvent_t asm_fork = nullptr, asm_join = nullptr, asm_join2 = nullptr;
  bem::KProf prof;      // BEM_OPT_KERNEL_TIMING

  // second stream and events of the lookahead LU (created on first use)
  cudaStream_t la_stream = nullptr;
  cudaEvent_t fork_event = nullptr;
  std::vector<cudaEvent_t> events;
  // third stream of the lookahead LU (thin updates)
  cudaStream_t thin_stream = nullptr;
  // Ensures 3*k events and the lookahead streams; false on failure.
  bool lookahead_ready(int k);

  // Grow-only device buffer for `slot` (NULL on allocation failure).
  void* get(int slot, size_t bytes);
  // Grow-only page-locked host staging buffer: a call's inputs go up and its
  // small results come back through it, one asynchronous copy each.  Growing
  // synchronizes the context's stream first (no copy from the old buffer is
  // in flight when it is freed).  NULL on allocation failure.
  char* pinned(size_t bytes);
  // marks the end of the last copy issued from the pinned buffer; pinned()
  // waits for it before handing the buffer out again
  void pin_issued();
  char* pin = nullptr;
  size_t pin_bytes = 0;
  cudaEvent_t pin_ev = nullptr;
  bool pin_pending = false;
  // timing events of the solve stages (created on first use)
  cudaEvent_t timing_event(int i);
  cudaEvent_t tev[6] = {};
  int cuda_fail(cudaError_t e, const char* where);
};

// Marks the context whose call runs on this thread (for kernel timing);
// collects the timings when the call returns (all streams synchronized).
struct CallScope {
  bem_ctx* c;
  explicit CallScope(bem_ctx* c_) : c(c_) { bem::tl_prof = (c && c->prof.on) ? &c->prof : nullptr; }
  ~CallScope() {
    if (bem::tl_prof) {
      if (c->la_stream) cudaStreamSynchronize(c->la_stream);
      cudaStreamSynchronize(c->stream);
      c->prof.collect();
    }
    bem::tl_prof = nullptr;
  }
};

int bem_check_geom(const bem_geom2d* g, int npg, double near_factor);
void bem_release_solver(bem_ctx* c);
// host-side rule tables of an assembly (element Gauss weights on the host)
void bem_build_rules(const bem_geom2d* g, int npg, const double* ew_host, bem::Rules& R);
// Stages the geometry on the device (host inputs: one copy through the
// pinned buffer, together with the nb boundary-condition codes and values
// when BC/BV are given; device inputs are used in place).
int bem_stage_geom(bem_ctx* c, const bem_geom2d* g, int npg, int mem, bem::GeomDev& gd,
                   bem::Rules& R, int64_t nb = 0, const int32_t* BC = nullptr, const double* BV = nullptr,
                   const int32_t** dBC = nullptr, const double** dBV = nullptr);
int bem_run_assembly(bem_ctx* c, bem::AsmRequest& q);
int bem_assemble_system_dev(bem_ctx* c, const bem_geom2d* g, const bem::Physics& ph,
                            const int32_t* BC, const double* BV, int npg, double nf, int mem,
                            int prec, double* A, int64_t lda, float* A32, double* b);
