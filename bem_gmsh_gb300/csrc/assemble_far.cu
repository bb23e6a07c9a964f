// Dense 2-D BEM influence-matrix assembly on sm_103a: far-field tiles.
//
// Restates `H_G_full_direct` (src/Core/Assembly_full.jl:61-175) of the
// reference, split the GB300 way:
//   far_kernel      one CTA per (collocation block x element block) tile.
//                   Element/node records of the tile are staged into shared
//                   memory by the bulk-copy engine (cp.async.bulk + mbarrier).
//                   Each thread owns 16 bytes of consecutive matrix rows and
//                   walks the tile's columns, so every warp store is one
//                   coalesced 512-byte column segment.  Far pairs get nodal
//                   lumping (`_far_nodal_scalar!`/`_far_nodal_vec!`,
//                   Assembly_full.jl:801-822); pairs that a conservative FP32
//                   bounding-box test calls possibly near are skipped.
//   near_classify_kernel  the same box test over all (point, element) pairs,
//                   ahead of the far kernel, lists the possibly-near pairs, so
//                   that the near kernel runs beside the far kernel.
//   near_kernel     one thread per listed pair: the exact FP64 near test
//                   (`_near_element`, :736-754), then the tanp3c near-singular
//                   integral, or FP64 far lumping if the pair is far after all.
//   singular_kernel one thread per boundary collocation node: interpolated
//                   Guiggiani on its own element (:397-457).
//   finalize_kernel the row-sum diagonal H_ii = -sum_{j!=i} H_ij (:384-390,
//                   :777-787), accumulated on the fly in FP64.
// Output is either (H, G) column-major, or the boundary-condition swap of
// `applyBC` (src/Core/Boundary_conditions.jl:54-75, 152-174) fused in: A and b.
#include "bem_device.cuh"
#include "bem_kernels.h"
#include "bem_prof.h"
#include "df32.cuh"

namespace bem {

// ---------------------------------------------------------------------------
// packing: FP32 hi/lo coordinates, per-node coefficients, per-element boxes
// ---------------------------------------------------------------------------
__device__ __forceinline__ void split_f(double v, float& hi, float& lo) {
  hi = (float)v;
  lo = (float)(v - (double)hi);
}

// row record: x_hi, x_lo, y_hi, y_lo
__global__ void pack_rows_kernel(GeomDev g, float4* rows) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.nt) return;
  float4 r;
  split_f(g.px[i], r.x, r.y);
  split_f(g.py[i], r.z, r.w);
  rows[i] = r;
}

// node record (32 B): x_hi, x_lo, y_hi, y_lo, nx, ny, cG, cH
// Laplace: G = log2(R2) * cG, H = (r.n) / R2 * cH
// Kelvin : cG = cH = J w (the weight only)
__global__ void pack_nodes_kernel(GeomDev g, Rules R, Physics ph, NodeRec* nodes) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= g.n) return;
  NodeRec r;
  split_f(g.px[j], r.xh, r.xl);
  split_f(g.py[j], r.yh, r.yl);
  r.nx = (float)g.nx[j];
  r.ny = (float)g.ny[j];
  double wjk = g.jac[j] * R.ew[j % g.nn];
  if (ph.kind == 0) {
    r.cG = (float)(-wjk * 0.6931471805599453 / (4 * kPi * ph.k));
    r.cH = (float)(wjk / (2 * kPi));
  } else {
    r.cG = (float)wjk;
    r.cH = (float)wjk;
  }
  nodes[j] = r;
}

// double-float log table (one thread per entry)
__global__ void logtab_kernel(float4* t) {
  const int i = threadIdx.x;
  if (i < df::kLogTable) {
    const df::LogEntry e = df::log_entry(i);
    t[i] = make_float4(e.rc_h, e.rc_l, e.lc_h, e.lc_l);
  }
}

// double-float node record (Laplace): G = log(R2) cG, H = (r.n) / R2 cH with
// the constants of laplace_UT times J w, and the boundary value of the node
__global__ void pack_nodes_df_kernel(GeomDev g, Rules R, Physics ph, const double* bv, NodeDF* nodes) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= g.n) return;
  NodeDF r;
  df::split3(g.px[j], r.xa, r.xb, r.xc);
  df::split3(g.py[j], r.ya, r.yb, r.yc);
  df::f2 t = df::from_double(g.nx[j]);
  r.nxh = t.h; r.nxl = t.l;
  t = df::from_double(g.ny[j]);
  r.nyh = t.h; r.nyl = t.l;
  const double wjk = g.jac[j] * R.ew[j % g.nn];
  const double inv2pi = 1.0 / (2 * kPi);
  t = df::from_double(-(0.5 * inv2pi / ph.k) * wjk);
  r.cGh = t.h; r.cGl = t.l;
  t = df::from_double(inv2pi * wjk);
  r.cHh = t.h; r.cHl = t.l;
  t = df::from_double(bv ? bv[j] : 0.0);
  r.bvh = t.h; r.bvl = t.l;
  nodes[j] = r;
}

// double-float node record (Kelvin): the constants of kelvin_UT times J w,
// cU = J w / (2 prod1 mu), cUl = -(3 - 4 nu) / 2 cU (the log(1/R) term as
// log(R2)), cT = -J w / prod1 with prod1 = 4 pi (1 - nu), and the node's two
// boundary values
__global__ void pack_nodes_dfk_kernel(GeomDev g, Rules R, Physics ph, const double* bv, NodeDFK* nodes) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= g.n) return;
  NodeDFK r;
  df::split3(g.px[j], r.xa, r.xb, r.xc);
  df::split3(g.py[j], r.ya, r.yb, r.yc);
  df::f2 t = df::from_double(g.nx[j]);
  r.nxh = t.h; r.nxl = t.l;
  t = df::from_double(g.ny[j]);
  r.nyh = t.h; r.nyl = t.l;
  const double wjk = g.jac[j] * R.ew[j % g.nn];
  const double prod1 = 4 * kPi * (1 - ph.nu);
  const double cU = wjk / (2 * prod1 * ph.mu);
  t = df::from_double(cU);
  r.cUh = t.h; r.cUl = t.l;
  t = df::from_double(-(3 - 4 * ph.nu) / 2 * cU);
  r.cLh = t.h; r.cLl = t.l;
  t = df::from_double(-wjk / prod1);
  r.cTh = t.h; r.cTl = t.l;
  t = df::from_double(bv ? bv[2 * j] : 0.0);
  r.bv0h = t.h; r.bv0l = t.l;
  t = df::from_double(bv ? bv[2 * j + 1] : 0.0);
  r.bv1h = t.h; r.bv1l = t.l;
  nodes[j] = r;
}

// element record (32 B): conservative box of the element's nodes and the
// squared near limit, widened so that a pair the box test calls far is far
// for the exact FP64 test as well.
// largest |coordinate| of the collocation points (non-negative doubles
// order like their bit patterns)
__global__ void absmax_kernel(GeomDev g, unsigned long long* out) {
  unsigned long long m = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.nt; i += gridDim.x * blockDim.x) {
    double v = fmax(fabs(g.px[i]), fabs(g.py[i]));
    m = max(m, (unsigned long long)__double_as_longlong(v));
  }
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// The margin covers the FP32 rounding of coordinates, box and distance
// (a few 2^-24 relative to the coordinate scale) with room to spare.
__global__ void pack_elems_kernel(GeomDev g, double near_factor, const unsigned long long* absmax,
                                  ElemRec* el) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.ne) return;
  const double abs_margin = 1e-6 * __longlong_as_double((long long)*absmax);
  double lox = INFINITY, loy = INFINITY, hix = -INFINITY, hiy = -INFINITY;
  for (int k = 0; k < g.nn; ++k) {
    double x = g.px[e * g.nn + k], y = g.py[e * g.nn + k];
    lox = fmin(lox, x);
    loy = fmin(loy, y);
    hix = fmax(hix, x);
    hiy = fmax(hiy, y);
  }
  double lim = near_factor * g.elen[e];
  double limw = lim * (1.0 + 1e-5) + abs_margin;
  ElemRec r;
  r.lox = __double2float_rd(lox);
  r.loy = __double2float_rd(loy);
  r.hix = __double2float_ru(hix);
  r.hiy = __double2float_ru(hiy);
  r.lim2 = (near_factor > 1e20) ? INFINITY : __double2float_ru(limw * limw);
  r.pad0 = r.pad1 = r.pad2 = 0.f;
  el[e] = r;
}

// Conservative box test of a source point (x, y) against an element record:
// true when the pair is far for the exact FP64 test as well.  Explicit
// round-to-nearest operations, so that the classification kernel and the far
// kernel agree bit for bit.
__device__ __forceinline__ bool box_far(float xh, float xl, float yh, float yl, const ElemRec& E) {
  const float x = __fadd_rn(xh, xl), y = __fadd_rn(yh, yl);
  const float dx = fmaxf(fmaxf(__fsub_rn(E.lox, x), __fsub_rn(x, E.hix)), 0.f);
  const float dy = fmaxf(fmaxf(__fsub_rn(E.loy, y), __fsub_rn(y, E.hiy)), 0.f);
  return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) > E.lim2;
}

// Possibly-near (point, element) pairs into the pair list: one thread per
// point, the CTA's 256 elements staged in shared memory.  Each warp first
// tests an element against the bounding box of its 32 points with the same
// operations: IEEE subtraction is monotonic, so a box distance above the
// limit means every point of the warp is far by the per-point test, and the
// 32 point tests are skipped.
__global__ void __launch_bounds__(256) near_classify_kernel(int nt, int ne, const float4* __restrict__ rows,
                                                            const ElemRec* __restrict__ elems,
                                                            int* pair_count, int2* pairs, int pair_cap) {
  __shared__ ElemRec s_e[256];
  const int i = blockIdx.x * 256 + threadIdx.x;
  const int e0 = blockIdx.y * 256;
  const int nel = min(256, ne - e0);
  if ((int)threadIdx.x < nel) s_e[threadIdx.x] = elems[e0 + threadIdx.x];
  __syncthreads();
  const bool valid = i < nt;
  const float4 r = rows[valid ? i : nt - 1];
  const int lane = threadIdx.x & 31;
  const float x = __fadd_rn(r.x, r.y), y = __fadd_rn(r.z, r.w);
  float bx0 = x, bx1 = x, by0 = y, by1 = y;
  for (int o = 16; o > 0; o >>= 1) {
    bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
    bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
    by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, o));
    by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, o));
  }
  for (int el = 0; el < nel; ++el) {
    const ElemRec E = s_e[el];
    const float dx = fmaxf(fmaxf(__fsub_rn(E.lox, bx1), __fsub_rn(bx0, E.hix)), 0.f);
    const float dy = fmaxf(fmaxf(__fsub_rn(E.loy, by1), __fsub_rn(by0, E.hiy)), 0.f);
    if (__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)) > E.lim2) continue;  // warp-uniform
    const bool need = valid && !box_far(r.x, r.y, r.z, r.w, E);
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(pair_count, __popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const int slot = base + __popc(m & ((1u << lane) - 1));
        if (slot < pair_cap) pairs[slot] = make_int2(i, e0 + el);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// bulk-copy staging helpers (TMA engine, non-tensor form)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait on phase 0 of the barrier.  Returns false on timeout.
__device__ __forceinline__ bool mbar_wait0(uint64_t* bar) {
  uint32_t done = 0;
  for (int it = 0; it < (1 << 22) && !done; ++it) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(0u)
        : "memory");
  }
  return done != 0;
}

// ---------------------------------------------------------------------------
// far kernel
// ---------------------------------------------------------------------------
template <typename T>
struct VecOf;
template <>
struct VecOf<float> {
  using type = float4;
  static constexpr int n = 4;
};
template <>
struct VecOf<double> {
  using type = double2;
  static constexpr int n = 2;
};

// FP32 kernel values for one (source, node) pair.  NC = 1 Laplace, 4 Kelvin.
template <int NC>
__device__ __forceinline__ void far_eval_f32(const Physics& ph, float rx, float ry, const NodeRec& nd,
                                             float* U, float* T) {
  float R2 = rx * rx + ry * ry;
  if constexpr (NC == 1) {
    U[0] = __log2f(R2) * nd.cG;
    T[0] = __fdividef(rx * nd.nx + ry * nd.ny, R2) * nd.cH;
  } else {
    float mu = (float)ph.mu, nu = (float)ph.nu;
    float invR = rsqrtf(R2);
    float dr1 = rx * invR, dr2 = ry * invR;
    float drdn = dr1 * nd.nx + dr2 * nd.ny;
    const float pi = 3.14159265358979f;
    float prod1 = 4.f * pi * (1.f - nu);
    float prod2 = (3.f - 4.f * nu) * (-0.5f * 0.69314718055994531f) * __log2f(R2);
    float ib = __fdividef(nd.cG, 2.f * prod1 * mu);
    U[0] = (prod2 + dr1 * dr1) * ib;
    U[1] = (dr1 * dr2) * ib;
    U[2] = U[1];
    U[3] = (prod2 + dr2 * dr2) * ib;
    float fat = __fdividef(invR, prod1) * nd.cH;
    float c = 1.f - 2.f * nu;
    T[0] = -drdn * (c + 2.f * (dr1 * dr1)) * fat;
    T[3] = -drdn * (c + 2.f * (dr2 * dr2)) * fat;
    T[1] = -(drdn * 2.f * dr1 * dr2 - c * (dr1 * nd.ny - dr2 * nd.nx)) * fat;
    T[2] = -(drdn * 2.f * dr1 * dr2 - c * (dr2 * nd.nx - dr1 * nd.ny)) * fat;
  }
}


// One launch computes the tile rows [row0, row0 + 32*SPT) of collocation
// points and the tile elements [e0, e0 + BE).  PREC: 0 = FP32 math and
// outputs, 1 = FP64 math and outputs, 2 = FP64 math with an FP64 and an FP32
// copy of A (mixed-precision solve).  FUSED: write A and accumulate b.
template <int NC, int PREC, bool FUSED>
__global__ void __launch_bounds__(256) far_kernel(FarArgs a) {
  using OutT = typename std::conditional<PREC == 0, float, double>::type;
  constexpr int DOF = (NC == 1) ? 1 : 2;
  constexpr int RPT = VecOf<OutT>::n;     // matrix rows per thread (16 B)
  constexpr int SPT = RPT / DOF;           // source points per thread
  constexpr int EL = 8;                    // element lanes
  constexpr int BE = 32;                   // elements per tile
  const int nn = a.nn;

  constexpr int NDB =
      (PREC == 3) ? (NC == 1 ? (int)sizeof(NodeDF) : (int)sizeof(NodeDFK)) : (int)sizeof(NodeRec);
  __shared__ __align__(16) ElemRec s_el[BE];
  __shared__ __align__(16) unsigned char s_ndraw[BE * BEM_MAXNN * NDB];
  __shared__ __align__(16) float4 s_log[PREC == 3 ? df::kLogTable : 1];
  __shared__ __align__(8) uint64_t s_bar;
  const NodeRec* s_nd = (const NodeRec*)s_ndraw;
  const NodeDF* s_ndf = (const NodeDF*)s_ndraw;
  const NodeDFK* s_ndk = (const NodeDFK*)s_ndraw;
  __shared__ double s_red[EL][32 * SPT * DOF * DOF];
  __shared__ double s_redb[EL][32 * SPT * DOF];

  const int tid = threadIdx.x;
  const int rg = tid & 31;      // row group
  const int lane_e = tid >> 5;  // element lane (warp id)
  const int src0 = blockIdx.x * 32 * SPT + rg * SPT;  // first source point
  const int e0 = blockIdx.y * BE;
  const int ne_t = min(BE, a.ne - e0);

  // ---- stage the tile's element and node records ----
  if (tid == 0) {
    mbar_init(&s_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if constexpr (PREC == 3) {
    for (int i = tid; i < df::kLogTable; i += blockDim.x) s_log[i] = a.logtab[i];
  }
  __syncthreads();
  if (tid == 0) {
    uint32_t eb = (uint32_t)(ne_t * sizeof(ElemRec));
    uint32_t nb = (uint32_t)(ne_t * nn * NDB);
    mbar_expect_tx(&s_bar, eb + nb);
    bulk_g2s(s_el, a.elems + e0, eb, &s_bar);
    if constexpr (PREC == 3)
      bulk_g2s(s_ndraw, (const unsigned char*)a.nodes_df + (size_t)e0 * nn * NDB, nb, &s_bar);
    else
      bulk_g2s(s_ndraw, a.nodes + (size_t)e0 * nn, nb, &s_bar);
  }
  // block-uniform decision: either every thread saw the copy land or the
  // whole CTA reports the timeout and leaves
  const int staged = __syncthreads_and(mbar_wait0(&s_bar) ? 1 : 0);
  if (!staged) {
    if (tid == 0) atomicOr(a.status, 1);
    return;
  }

  // ---- source points of this thread ----
  float sxh[SPT], sxl[SPT], syh[SPT], syl[SPT];
  double sx[SPT], sy[SPT];
  bool valid[SPT];
#pragma unroll
  for (int s = 0; s < SPT; ++s) {
    int i = src0 + s;
    valid[s] = i < a.nt;
    int ic = valid[s] ? i : a.nt - 1;
    float4 r = a.rows[ic];
    sxh[s] = r.x; sxl[s] = r.y; syh[s] = r.z; syl[s] = r.w;
    if constexpr (PREC != 0) {
      sx[s] = a.px[ic];
      sy[s] = a.py[ic];
    }
  }
  // double-float state: three-float source coordinates, row sums and b
  float s3x[PREC == 3 ? SPT : 1][3], s3y[PREC == 3 ? SPT : 1][3];
  df::f2 rs_df[PREC == 3 ? SPT * DOF * DOF : 1], b_df[PREC == 3 ? SPT * DOF : 1];
  if constexpr (PREC == 3) {
#pragma unroll
    for (int s = 0; s < SPT; ++s) {
      df::split3(sx[s], s3x[s][0], s3x[s][1], s3x[s][2]);
      df::split3(sy[s], s3y[s][0], s3y[s][1], s3y[s][2]);
    }
#pragma unroll
    for (int r = 0; r < SPT * DOF * DOF; ++r) rs_df[r] = df::f2{0.f, 0.f};
#pragma unroll
    for (int r = 0; r < SPT * DOF; ++r) b_df[r] = df::f2{0.f, 0.f};
  }

  double rowsum[SPT * DOF][DOF];  // [row][column dof]
  double bacc[SPT * DOF];
#pragma unroll
  for (int r = 0; r < SPT * DOF; ++r) {
    bacc[r] = 0.0;
#pragma unroll
    for (int b = 0; b < DOF; ++b) rowsum[r][b] = 0.0;
  }
  // FP32 H, G: the row sums in FP32 pairs (an FP64 add and conversion per
  // entry would make GB300's FP64 pipe the kernel's bound)
  df::f2 rs32[PREC == 0 ? SPT * DOF * DOF : 1];
  if constexpr (PREC == 0) {
#pragma unroll
    for (int r = 0; r < SPT * DOF * DOF; ++r) rs32[r] = df::f2{0.f, 0.f};
  }

  const size_t ld = (size_t)a.ld;
  const size_t ldg = (size_t)a.ldg;
  const bool vec_ok = a.vec_ok && (src0 + SPT <= a.nt);

  for (int el = lane_e; el < ne_t; el += EL) {
    const ElemRec E = s_el[el];
    const int e = e0 + el;
    // conservative box test per source point (the possibly-near pairs are
    // listed by near_classify_kernel with the same test)
    bool far[SPT];
#pragma unroll
    for (int s = 0; s < SPT; ++s) far[s] = box_far(sxh[s], sxl[s], syh[s], syl[s], E) || !valid[s];
    if constexpr (PREC == 3 && NC == 4) {
      static_assert(FUSED && SPT == 1, "double-float Kelvin far field: fused, one source point per thread");
      const df::LogEntry* tab = (const df::LogEntry*)s_log;
      const df::f2 cc{a.c1h, a.c1l};
      for (int k = 0; k < nn; ++k) {
        const NodeDFK nd = s_ndk[el * nn + k];
        const int j = e * nn + k;
        df::f2 U[4], T[4];
        if (far[0]) {
          const df::f2 rx = df::diff3(nd.xa, nd.xb, nd.xc, s3x[0][0], s3x[0][1], s3x[0][2]);
          const df::f2 ry = df::diff3(nd.ya, nd.yb, nd.yc, s3y[0][0], s3y[0][1], s3y[0][2]);
          const df::f2 R2 = df::add(df::sqr(rx), df::sqr(ry));
          const df::f2 inv = df::div(df::f2{1.f, 0.f}, R2);
          const df::f2 lg = df::log(R2, tab);
          const df::f2 nxd{nd.nxh, nd.nxl}, nyd{nd.nyh, nd.nyl};
          const df::f2 cU{nd.cUh, nd.cUl}, cL{nd.cLh, nd.cLl}, cT{nd.cTh, nd.cTl};
          const df::f2 qxx = df::mul(df::sqr(rx), inv), qyy = df::mul(df::sqr(ry), inv);
          const df::f2 qxy = df::mul(df::mul(rx, ry), inv);
          const df::f2 rn = df::add(df::mul(rx, nxd), df::mul(ry, nyd));
          const df::f2 ul = df::mul(cL, lg);
          U[0] = df::add(ul, df::mul(cU, qxx));
          U[1] = df::mul(cU, qxy);
          U[2] = U[1];
          U[3] = df::add(ul, df::mul(cU, qyy));
          const df::f2 sT = df::mul(cT, df::mul(rn, inv));
          T[0] = df::mul(sT, df::add(cc, df::add(qxx, qxx)));
          T[3] = df::mul(sT, df::add(cc, df::add(qyy, qyy)));
          const df::f2 cti = df::mul(cT, inv);
          const df::f2 t2 = df::mul(df::add(rn, rn), qxy);
          const df::f2 tw = df::mul(cc, df::add(df::mul(rx, nyd), df::neg(df::mul(ry, nxd))));
          T[1] = df::mul(cti, df::add(t2, df::neg(tw)));
          T[2] = df::mul(cti, df::add(t2, tw));
        } else {
#pragma unroll
          for (int c = 0; c < 4; ++c) U[c] = T[c] = df::f2{0.f, 0.f};
        }
#pragma unroll
        for (int b = 0; b < 2; ++b) {
          const int col = 2 * j + b;
          const bool gcol = a.bc[col] == 0;  // column takes -G and b takes -H bv
          const df::f2 bvv = b == 0 ? df::f2{nd.bv0h, nd.bv0l} : df::f2{nd.bv1h, nd.bv1l};
          const df::f2 bvs = gcol ? df::neg(bvv) : bvv;
          double av[2];
#pragma unroll
          for (int ar = 0; ar < 2; ++ar) {
            const df::f2 Tv = T[ar * 2 + b], Uv = U[ar * 2 + b];
            rs_df[ar * 2 + b] = df::add(rs_df[ar * 2 + b], Tv);
            b_df[ar] = df::add(b_df[ar], df::mul(gcol ? Tv : Uv, bvs));
            av[ar] = df::to_double(gcol ? df::neg(Uv) : Tv);
          }
          if (far[0] && valid[0]) {
            double* Ac = (double*)a.H + (size_t)src0 * 2 + (size_t)col * ld;
            if (vec_ok) {
              *(double2*)Ac = make_double2(av[0], av[1]);
            } else {
              Ac[0] = av[0];
              Ac[1] = av[1];
            }
          }
        }
      }
      continue;
    }
    if constexpr (PREC == 3 && NC == 1) {
      static_assert(FUSED, "double-float far field: fused systems only");
      const df::LogEntry* tab = (const df::LogEntry*)s_log;
      for (int k = 0; k < nn; ++k) {
        const NodeDF nd = s_ndf[el * nn + k];
        const int j = e * nn + k;
        const bool gcol = a.bc[j] == 0;  // column takes -G and b takes -H bv
        const df::f2 cG{nd.cGh, nd.cGl}, cH{nd.cHh, nd.cHl};
        const df::f2 nxd{nd.nxh, nd.nxl}, nyd{nd.nyh, nd.nyl};
        const df::f2 bvv = gcol ? df::f2{-nd.bvh, -nd.bvl} : df::f2{nd.bvh, nd.bvl};
        double av[SPT];
#pragma unroll
        for (int s = 0; s < SPT; ++s) {
          df::f2 Hs{0.f, 0.f}, Gs{0.f, 0.f};
          if (far[s]) {
            const df::f2 rx = df::diff3(nd.xa, nd.xb, nd.xc, s3x[s][0], s3x[s][1], s3x[s][2]);
            const df::f2 ry = df::diff3(nd.ya, nd.yb, nd.yc, s3y[s][0], s3y[s][1], s3y[s][2]);
            const df::f2 R2 = df::add(df::sqr(rx), df::sqr(ry));
            Gs = df::mul(df::log(R2, tab), cG);
            const df::f2 num = df::add(df::mul(rx, nxd), df::mul(ry, nyd));
            Hs = df::mul(df::div(num, R2), cH);
          }
          rs_df[s] = df::add(rs_df[s], Hs);
          b_df[s] = df::add(b_df[s], df::mul(gcol ? Hs : Gs, bvv));
          av[s] = df::to_double(gcol ? df::neg(Gs) : Hs);
        }
        // only far entries are stored: near and on-element entries belong to
        // the near and singular kernels, which may run concurrently
        double* Ac = (double*)a.H + (size_t)src0 + (size_t)j * ld;
        if (vec_ok && far[0] && far[1]) {
          *(double2*)Ac = make_double2(av[0], av[1]);
        } else {
#pragma unroll
          for (int s = 0; s < SPT; ++s)
            if (far[s] && src0 + s < a.nt) Ac[s] = av[s];
        }
      }
      continue;
    }
    for (int k = 0; k < nn; ++k) {
      const NodeRec nd = s_nd[el * nn + k];
      const int j = e * nn + k;
      OutT hv[DOF][SPT * DOF], gv[DOF][SPT * DOF];  // [column dof b][row]
#pragma unroll
      for (int s = 0; s < SPT; ++s) {
        if constexpr (PREC == 0) {
          float rx = (nd.xh - sxh[s]) + (nd.xl - sxl[s]);
          float ry = (nd.yh - syh[s]) + (nd.yl - syl[s]);
          float U[NC], Tk[NC];
          far_eval_f32<NC>(a.ph, rx, ry, nd, U, Tk);
#pragma unroll
          for (int ar = 0; ar < DOF; ++ar)
#pragma unroll
            for (int b = 0; b < DOF; ++b) {
              hv[b][s * DOF + ar] = far[s] ? Tk[ar * DOF + b] : 0.f;
              gv[b][s * DOF + ar] = far[s] ? U[ar * DOF + b] : 0.f;
            }
        } else {
          double U[NC], Tk[NC];
          if (far[s]) {
            far_eval_f64<NC>(a.ph, a.px[j] - sx[s], a.py[j] - sy[s], a.nx[j], a.ny[j],
                             a.jac[j] * a.ew[k], U, Tk);
          } else {
#pragma unroll
            for (int c = 0; c < NC; ++c) U[c] = Tk[c] = 0.0;
          }
#pragma unroll
          for (int ar = 0; ar < DOF; ++ar)
#pragma unroll
            for (int b = 0; b < DOF; ++b) {
              hv[b][s * DOF + ar] = Tk[ar * DOF + b];
              gv[b][s * DOF + ar] = U[ar * DOF + b];
            }
        }
      }
      // accumulate row sums (and b), then store
#pragma unroll
      for (int b = 0; b < DOF; ++b) {
        const int col = DOF * j + b;
        double bvj = 0.0;
        int bcj = 1;
        if constexpr (FUSED) {
          bcj = a.bc[col];
          bvj = a.bv[col];
        }
#pragma unroll
        for (int r = 0; r < SPT * DOF; ++r) {
          if constexpr (PREC == 0)
            rs32[r * DOF + b] = df::add_f(rs32[r * DOF + b], (float)hv[b][r]);
          else
            rowsum[r][b] += (double)hv[b][r];
          if constexpr (FUSED) bacc[r] += (bcj == 0) ? -(double)hv[b][r] * bvj : (double)gv[b][r] * bvj;
        }
        const size_t row0 = (size_t)src0 * DOF;
        // only far entries are stored (see the double-float branch)
        bool allfar = true;
#pragma unroll
        for (int s = 0; s < SPT; ++s) allfar = allfar && far[s];
        if constexpr (!FUSED) {
          OutT* Hc = (OutT*)a.H + row0 + (size_t)col * ld;
          OutT* Gc = (OutT*)a.G + row0 + (size_t)col * ldg;
          if (vec_ok && allfar) {
            typename VecOf<OutT>::type hvv, gvv;
            OutT* hp = (OutT*)&hvv;
            OutT* gp = (OutT*)&gvv;
#pragma unroll
            for (int r = 0; r < RPT; ++r) { hp[r] = hv[b][r]; gp[r] = gv[b][r]; }
            *(typename VecOf<OutT>::type*)Hc = hvv;
            *(typename VecOf<OutT>::type*)Gc = gvv;
          } else {
#pragma unroll
            for (int r = 0; r < RPT; ++r)
              if (far[r / DOF] && src0 + r / DOF < a.nt) { Hc[r] = hv[b][r]; Gc[r] = gv[b][r]; }
          }
        } else {
          OutT* Ac = (OutT*)a.H + row0 + (size_t)col * ld;
          OutT av[RPT];
#pragma unroll
          for (int r = 0; r < RPT; ++r) av[r] = (bcj == 0) ? -gv[b][r] : hv[b][r];
          if (vec_ok && allfar) {
            typename VecOf<OutT>::type v;
            OutT* vp = (OutT*)&v;
#pragma unroll
            for (int r = 0; r < RPT; ++r) vp[r] = av[r];
            *(typename VecOf<OutT>::type*)Ac = v;
            if constexpr (PREC == 2) {
              float* A32 = a.A32 + row0 + (size_t)col * ld;
              *(float2*)A32 = make_float2((float)av[0], (float)av[1]);
            }
          } else {
#pragma unroll
            for (int r = 0; r < RPT; ++r)
              if (far[r / DOF] && src0 + r / DOF < a.nt) {
                Ac[r] = av[r];
                if constexpr (PREC == 2) a.A32[row0 + r + (size_t)col * ld] = (float)av[r];
              }
          }
        }
      }
    }
  }
  if constexpr (PREC == 3) {
#pragma unroll
    for (int r = 0; r < SPT * DOF; ++r) {
#pragma unroll
      for (int b = 0; b < DOF; ++b)
        rowsum[r][b] = (double)rs_df[r * DOF + b].h + (double)rs_df[r * DOF + b].l;
      bacc[r] = (double)b_df[r].h + (double)b_df[r].l;
    }
  }
  if constexpr (PREC == 0) {
#pragma unroll
    for (int r = 0; r < SPT * DOF; ++r)
#pragma unroll
      for (int b = 0; b < DOF; ++b)
        rowsum[r][b] = (double)rs32[r * DOF + b].h + (double)rs32[r * DOF + b].l;
  }
  // reduce row sums across element lanes, one FP64 atomic per row
#pragma unroll
  for (int r = 0; r < SPT * DOF; ++r) {
#pragma unroll
    for (int b = 0; b < DOF; ++b) s_red[lane_e][(rg * SPT * DOF + r) * DOF + b] = rowsum[r][b];
    if constexpr (FUSED) s_redb[lane_e][rg * SPT * DOF + r] = bacc[r];
  }
  __syncthreads();
  for (int t = tid; t < 32 * SPT * DOF * DOF; t += blockDim.x) {
    double s = 0.0;
#pragma unroll
    for (int l = 0; l < EL; ++l) s += s_red[l][t];
    size_t idx = (size_t)blockIdx.x * 32 * SPT * DOF * DOF + t;  // row * DOF + b
    if (idx < (size_t)a.nt * DOF * DOF) atomicAdd(a.rowsum + idx, s);
  }
  if constexpr (FUSED) {
    for (int t = tid; t < 32 * SPT * DOF; t += blockDim.x) {
      double sb = 0.0;
#pragma unroll
      for (int l = 0; l < EL; ++l) sb += s_redb[l][t];
      int row = blockIdx.x * 32 * SPT * DOF + t;
      if (row < a.nt * DOF) atomicAdd(a.b + row, sb);
    }
  }
}

}  // namespace bem

// ---------------------------------------------------------------------------
// host launcher
// ---------------------------------------------------------------------------
namespace bem {

template <int NC, int PREC, bool FUSED>
static void launch_variant(const AsmRequest& q, cudaStream_t st) {
  using OutT = typename std::conditional<PREC == 0, float, double>::type;
  constexpr int DOF = (NC == 1) ? 1 : 2;
  constexpr bool MIXED = (PREC == 2);
  const GeomDev& g = q.g;
  FarArgs fa{};
  fa.nt = g.nt; fa.n = g.n; fa.ne = g.ne; fa.nn = g.nn;
  fa.ld = q.ld; fa.ldg = q.ldg;
  constexpr int RPT = 16 / sizeof(OutT);
  fa.vec_ok = (q.ld % RPT == 0) && (FUSED || q.ldg % RPT == 0) &&
              (((uintptr_t)q.H) % 16 == 0) && (FUSED || ((uintptr_t)q.G) % 16 == 0) &&
              (!MIXED || ((uintptr_t)q.A32) % 16 == 0);
  fa.pair_cap = q.pair_cap;
  fa.ph = q.ph;
  fa.rows = q.rows; fa.nodes = q.nodes; fa.elems = q.elems;
  fa.nodes_df = q.nodes_df; fa.logtab = q.logtab;
  if constexpr (PREC == 3) {
    logtab_kernel<<<1, 160, 0, st>>>(q.logtab);
    if constexpr (NC == 1) {
      pack_nodes_df_kernel<<<(g.n + 255) / 256, 256, 0, st>>>(g, q.R, q.ph, q.bv, q.nodes_df);
    } else {
      pack_nodes_dfk_kernel<<<(g.n + 255) / 256, 256, 0, st>>>(g, q.R, q.ph, q.bv, (NodeDFK*)q.nodes_df);
      const df::f2 c1 = df::from_double(1 - 2 * q.ph.nu);
      fa.c1h = c1.h;
      fa.c1l = c1.l;
    }
    count_launches(2);
  }
  fa.px = g.px; fa.py = g.py; fa.nx = g.nx; fa.ny = g.ny; fa.jac = g.jac;
  for (int k = 0; k < BEM_MAXNN; ++k) fa.ew[k] = q.R.ew[k];
  fa.H = q.H; fa.G = q.G; fa.A32 = q.A32;
  fa.bc = q.bc; fa.bv = q.bv; fa.b = q.b;
  fa.rowsum = q.rowsum;
  fa.pair_count = q.counters;
  fa.pairs = q.pairs;
  fa.status = q.counters + 1;
  NearArgs na{};
  na.g = g; na.R = q.R; na.ph = q.ph; na.near_factor = q.near_factor;
  na.ld = q.ld; na.ldg = q.ldg; na.pair_cap = q.pair_cap;
  na.pair_count = q.counters; na.pairs = q.pairs;
  na.H = q.H; na.G = q.G; na.A32 = q.A32;
  na.bc = q.bc; na.bv = q.bv; na.b = q.b; na.rowsum = q.rowsum; na.gdiag = q.gdiag;
  na.mode = PREC == 0 ? 0 : (!FUSED ? 1 : (MIXED ? 3 : 2));  // PREC 3: fused FP64 (2)

  FinalArgs fi{};
  fi.nt = g.nt; fi.n = g.n; fi.ld = q.ld; fi.H = q.H; fi.A32 = q.A32;
  fi.bc = q.bc; fi.bv = q.bv; fi.b = q.b; fi.rowsum = q.rowsum; fi.gdiag = q.gdiag;
  fi.mode = na.mode;

  // the on-element rows need neither the far results nor the pair list: on
  // a side stream they run beside the far and near kernels (every kernel
  // writes its own entries; row sums are atomic)
  {
    KScope ks(st, KC_NEAR);
    dim3 cg((g.nt + 255) / 256, (g.ne + 255) / 256);
    near_classify_kernel<<<cg, 256, 0, st>>>(g.nt, g.ne, q.rows, q.elems, q.counters, q.pairs, q.pair_cap);
  }
  const bool side = q.aux != nullptr && g.n > 0;
  const bool side2 = side && q.aux2 != nullptr;
  if (side) {
    cudaEventRecord(q.ev_fork, st);
    cudaStreamWaitEvent(q.aux, q.ev_fork, 0);
    launch_singular(na, NC, g.n, q.aux);
    cudaEventRecord(q.ev_join, q.aux);
  }
  if (side2) {
    // the near pairs (FP64 pipe) beside the far kernel (FP32 pipe)
    cudaStreamWaitEvent(q.aux2, q.ev_fork, 0);
    {
      KScope ks(q.aux2, KC_NEAR);
      launch_near_pairs(na, NC, q.aux2);
    }
    cudaEventRecord(q.ev_join2, q.aux2);
  }
  constexpr int SPT = RPT / DOF;
  dim3 grid((g.nt + 32 * SPT - 1) / (32 * SPT), (g.ne + 31) / 32);
  {
    KScope ks(st, KC_FAR);
    far_kernel<NC, PREC, FUSED><<<grid, 256, 0, st>>>(fa);
  }
  {
    KScope ks(st, KC_NEAR);
    if (!side2) launch_near_pairs(na, NC, st);
    if (!side) launch_singular(na, NC, g.n, st);
    if (side) cudaStreamWaitEvent(st, q.ev_join, 0);
    if (side2) cudaStreamWaitEvent(st, q.ev_join2, 0);
    launch_finalize(fi, NC, g.nt, st);
  }
  count_launches(g.n > 0 ? 9 : 8);
}

int launch_assembly(const AsmRequest& q, cudaStream_t st) {
  const GeomDev& g = q.g;
  const int dof = q.ph.kind == 0 ? 1 : 2;
  if (g.nt <= 0 || g.n <= 0 || g.ne <= 0) return (int)cudaErrorInvalidValue;
  cudaMemsetAsync(q.rowsum, 0, sizeof(double) * (size_t)g.nt * dof * dof, st);
  cudaMemsetAsync(q.counters, 0, 2 * sizeof(int), st);
  if (q.fused) cudaMemsetAsync(q.b, 0, sizeof(double) * (size_t)g.nt * dof, st);
  // columns of internal points: zero except the diagonal (finalize)
  if (g.nt > g.n) {
    size_t esz = (q.prec == 0) ? 4 : 8;
    size_t off = (size_t)dof * g.n * (size_t)q.ld;
    size_t cnt = (size_t)dof * (g.nt - g.n) * (size_t)q.ld;
    cudaMemsetAsync((char*)q.H + off * esz, 0, cnt * esz, st);
    if (q.prec == 2) cudaMemsetAsync(q.A32 + off, 0, cnt * 4, st);
  }
  pack_rows_kernel<<<(g.nt + 255) / 256, 256, 0, st>>>(g, q.rows);
  pack_nodes_kernel<<<(g.n + 255) / 256, 256, 0, st>>>(g, q.R, q.ph, q.nodes);
  cudaMemsetAsync(q.absmax, 0, sizeof(unsigned long long), st);
  absmax_kernel<<<64, 256, 0, st>>>(g, q.absmax);
  pack_elems_kernel<<<(g.ne + 255) / 256, 256, 0, st>>>(g, q.near_factor, q.absmax, q.elems);
  const int key = q.ph.kind * 100 + q.prec * 10 + q.fused;
  switch (key) {
    case 0: launch_variant<1, 0, false>(q, st); break;
    case 10: launch_variant<1, 1, false>(q, st); break;
    case 11: launch_variant<1, 1, true>(q, st); break;
    case 21: launch_variant<1, 2, true>(q, st); break;
    case 31: launch_variant<1, 3, true>(q, st); break;
    case 100: launch_variant<4, 0, false>(q, st); break;
    case 110: launch_variant<4, 1, false>(q, st); break;
    case 111: launch_variant<4, 1, true>(q, st); break;
    case 121: launch_variant<4, 2, true>(q, st); break;
    case 131: launch_variant<4, 3, true>(q, st); break;
    default: return (int)cudaErrorInvalidValue;
  }
  return (int)cudaGetLastError();
}

}  // namespace bem
