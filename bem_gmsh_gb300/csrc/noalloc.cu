// Allocation-free Laplace assembly: the scratch of the assembly lives in a
// file-scope device array instead of device memory obtained from cudaMalloc.
//
// For callers that cannot allocate device memory while they run: a host
// program whose device memory is owned by another allocator's pool (Julia's
// CUDA.jl or PyTorch caching allocators hold most of the device, so a
// cudaMalloc behind their back can fail or fragment it), a real-time or
// safety-critical loop that may only allocate during start-up, or code that
// runs where cudaMalloc is not permitted.  The caller passes inputs and
// outputs in device memory; this file owns everything else.
//
// The array is part of the library's device image: every GPU on which the
// library is used holds it (NOALLOC_BYTES) until the process exits.  Its
// device address is looked up once per device with cudaGetSymbolAddress the
// first time the entry point runs on that device (that first call loads the
// module and should happen before any stream capture).  Every call uses the
// same array, so two calls whose work overlaps on the GPU -- different
// streams, or different host threads on the same device -- race and corrupt
// each other's results; serialize them.  The parts that must start at zero
// (pair counter, row sums, status) are cleared on the stream by every call.
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/bem_gb300.h"
#include "bem_abi_internal.h"
#include "bem_kernels.h"

namespace {

constexpr int kMaxNt = BEM_NOALLOC_MAX_NT;  // collocation points
constexpr int kMaxNe = BEM_NOALLOC_MAX_NE;  // elements
constexpr int kPairCap = 24 * kMaxNt;       // near-pair list entries

constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kOffRows = 0;
constexpr size_t kOffNodes = align256(kOffRows + sizeof(float4) * kMaxNt);
constexpr size_t kOffElems = align256(kOffNodes + sizeof(bem::NodeRec) * kMaxNt);
constexpr size_t kOffRowsum = align256(kOffElems + sizeof(bem::ElemRec) * kMaxNe);
constexpr size_t kOffGdiag = align256(kOffRowsum + sizeof(double) * kMaxNt);
constexpr size_t kOffCounters = align256(kOffGdiag + sizeof(double) * kMaxNt);
constexpr size_t kOffPairs = align256(kOffCounters + 64);
constexpr size_t kBytes = align256(kOffPairs + sizeof(int2) * (size_t)kPairCap);
static_assert(kBytes == BEM_NOALLOC_BYTES, "BEM_NOALLOC_BYTES must match the scratch layout");

static __device__ __align__(256) unsigned char g_scratch[kBytes];

std::mutex g_mu;
void* g_addr[256] = {nullptr};

// device address of g_scratch on the current device (set-up on first use)
int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return BEM_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return BEM_ERR_CUDA;
    }
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return BEM_OK;
}

}  // namespace

extern "C" int bem_assemble_laplace2d_noalloc(const bem_geom2d* geom, double k, int npg,
                                              double near_factor, int dtype, void* H, int64_t ldh,
                                              void* G, int64_t ldg, void* cuda_stream) {
  int rc = bem_check_geom(geom, npg, near_factor);
  if (rc) return rc;
  if (geom->nt > kMaxNt || geom->ne > kMaxNe) return BEM_ERR_UNSUPPORTED;
  if (!(k > 0)) return BEM_ERR_INVALID;
  if (dtype != BEM_F32 && dtype != BEM_F64) return BEM_ERR_INVALID;
  if (!H || !G || ldh < geom->nt || ldg < geom->nt) return BEM_ERR_INVALID;
  cudaStream_t st = (cudaStream_t)cuda_stream;
  unsigned char* base = nullptr;
  rc = scratch_address((void**)&base);
  if (rc) return rc;

  bem::AsmRequest q{};
  // The element weights are read on the caller's stream, so that the read is
  // ordered after whatever the caller's earlier work on that stream wrote
  // (the weights feed the host-built quadrature tables).
  double ew[BEM_MAXNN];
  if (cudaMemcpyAsync(ew, geom->elem_weight, sizeof(double) * (geom->p + 1), cudaMemcpyDeviceToHost,
                      st) != cudaSuccess)
    return BEM_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return BEM_ERR_CUDA;
  bem_build_rules(geom, npg, ew, q.R);
  q.g.nt = geom->nt;
  q.g.n = geom->n;
  q.g.ne = geom->ne;
  q.g.nn = geom->p + 1;
  q.g.ngeo = geom->ngeo;
  q.g.px = geom->px;
  q.g.py = geom->py;
  q.g.nx = geom->nx;
  q.g.ny = geom->ny;
  q.g.jac = geom->jac;
  q.g.elen = geom->elen;
  q.g.gx = geom->geo_x;
  q.g.gy = geom->geo_y;
  q.ph.kind = 0;
  q.ph.k = k;
  q.near_factor = near_factor;
  q.prec = dtype == BEM_F32 ? 0 : 1;
  q.fused = 0;
  q.H = H;
  q.ld = ldh;
  q.G = G;
  q.ldg = ldg;
  q.rows = (float4*)(base + kOffRows);
  q.nodes = (bem::NodeRec*)(base + kOffNodes);
  q.elems = (bem::ElemRec*)(base + kOffElems);
  q.rowsum = (double*)(base + kOffRowsum);
  q.gdiag = (double*)(base + kOffGdiag);
  q.counters = (int*)(base + kOffCounters);
  q.absmax = (unsigned long long*)(base + kOffCounters + 32);
  q.pairs = (int2*)(base + kOffPairs);
  q.pair_cap = kPairCap;
  int lrc = bem::launch_assembly(q, st);
  if (lrc) return BEM_ERR_CUDA;
  int hc[2] = {0, 0};
  if (cudaMemcpyAsync(hc, q.counters, sizeof(hc), cudaMemcpyDeviceToHost, st) != cudaSuccess)
    return BEM_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return BEM_ERR_CUDA;
  if (hc[1] != 0) return BEM_ERR_INTERNAL;
  if (hc[0] > kPairCap) return BEM_ERR_UNSUPPORTED;  // more near pairs than the fixed list holds
  return BEM_OK;
}
