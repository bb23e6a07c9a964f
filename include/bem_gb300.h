/*
 * bem_gb300.h -- C ABI of the GB300-native dense 2-D BEM collocation path.
 *
 * Drop-in for the GPU slot of the Julia package `BEM` (l-s-campos/BEM_gmsh):
 * `assemble!(dad; method=:gpu)` dispatches to `H_G_gpu`
 * (src/Core/Assembly_full.jl:112-113), and `solve(dad)` runs `applyBC` +
 * `bem_linsolve` (src/Core/Solver.jl:24-64, 114-131).  Every entry point
 * takes plain pointers and sizes, returns an int status (0 = success) and
 * never throws.  Matrices are column-major (Julia `Matrix` layout) with an
 * explicit leading dimension, so a `ccall` can write into Julia arrays in
 * place.  Paths in comments are relative to the reference project root.
 *
 * Layout of a problem (what `format2d` builds, src/Core/Input.jl:136-197):
 *   - ne discontinuous elements of degree p; element e owns the boundary
 *     collocation nodes e*(p+1) .. e*(p+1)+p (0-based);
 *   - nt collocation points: the n = ne*(p+1) boundary nodes, then nt-n
 *     internal points;
 *   - Laplace: H is nt x nt, G is nt x n; Kelvin: H is 2nt x 2nt, G is
 *     2nt x 2n, degrees of freedom node-major (2i, 2i+1).
 */
#ifndef BEM_GB300_H
#define BEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define BEM_OK 0
#define BEM_ERR_INVALID 1       /* bad argument (ArgumentError in the reference) */
#define BEM_ERR_CUDA 2          /* CUDA runtime error, see bem_last_error() */
#define BEM_ERR_NOMEM 3         /* device allocation failed */
#define BEM_ERR_NOT_CONVERGED 4 /* refinement hit its iteration cap */
#define BEM_ERR_INTERNAL 5      /* a device-side wait timed out */
#define BEM_ERR_UNSUPPORTED 6   /* size/degree outside the compiled limits */

/* element type of matrix outputs */
#define BEM_F32 32
#define BEM_F64 64

/* where the pointers of a call live */
#define BEM_MEM_HOST 0
#define BEM_MEM_DEVICE 1

/* context options (bem_ctx_set_option) */
#define BEM_OPT_TCGEN05 1       /* LU trailing updates: 2 (default) a persistent warp-specialized tcgen05
                                   kernel (TMEM double buffer, C through TMA); 1 tcgen05, one CTA per
                                   tile; 0 legacy mma.sync */
#define BEM_OPT_KERNEL_TIMING 2 /* 1: time kernel classes with CUDA events (bem_kernel_times) */
#define BEM_OPT_FAR_DF 3        /* far-field Laplace entries of FP64 systems evaluated in double-float
                                   (FP32 pairs, ~1e-14 relative): 0 never, 1 (default) in mixed-precision
                                   solves, 2 also in bem_assemble_system2d.  Laplace and Kelvin. */
#define BEM_OPT_GRAPHS 4        /* 1 (default): the mixed solve's factorization (equilibration, look-ahead
                                   LU, sweep couplings) is captured in a CUDA graph on the second call with
                                   unchanged buffers and replayed; 0: direct launches.  Not used while
                                   BEM_OPT_KERNEL_TIMING is on. */
#define BEM_OPT_PIVOT_FALLBACK 5 /* 1 (default): a mixed solve whose FP32 LU (no pivoting) meets a
                                   vanishing pivot, or whose refinement stagnates above the FP64
                                   rounding floor (a restart cycle that does not halve the residual),
                                   is solved again by LU with partial pivoting in FP64 (the LAPACK
                                   getrf semantics of `bem_linsolve`), stats->pivoted = 1; 0: such a
                                   solve returns BEM_ERR_NOT_CONVERGED.  Reaching max_iter alone
                                   always returns BEM_ERR_NOT_CONVERGED. */
#define BEM_OPT_WAIT_LIMIT 6    /* polls before a device-side wait of the triangular sweeps gives up
                                   and the call returns BEM_ERR_INTERNAL (default 1 << 20, >= 1) */
#define BEM_OPT_INJECT 7        /* failure injection for tests, host side (default 0, or the value of
                                   the environment variable BEM_INJECT when the context is created):
                                   bit 0: every workspace allocation fails (BEM_ERR_NOMEM); bit 1: the
                                   triangular sweeps publish their results under another epoch than
                                   the one their readers wait for, so those bounded waits run out
                                   (BEM_ERR_INTERNAL, the context stays usable) */
#define BEM_OPT_NEARFIELD 8     /* near-singular map of the element integrals, the reference's `nearfield`
                                   knob (src/Core/Integration.jl:41-93, set per problem with set_cache!):
                                   0 (default) tanp3c, 1 plain Gauss rule, 2 euclid (sinh about the
                                   closest point, b = d / L), 3 csinh (sinh on the complex pole, eq. 40),
                                   4 sinhsinh (iterated sinh-sinh), 5 tangent (eq. 41), 6 complete cubic
                                   p3c; other values return BEM_ERR_INVALID */
#define BEM_OPT_SINGULAR 9      /* on-element rule, the reference's `singular` knob
                                   (src/Core/Assembly_full.jl:282-283): 0 (default) interpolated
                                   Guiggiani, 1 Telles cubic map of the npg Gauss rule */
#define BEM_OPT_SWEEP_CTAS 11   /* CTAs per block row of the preconditioner's triangular sweeps (1..4, default
                                   4; at most what the GPU keeps resident): helpers sum the block row's
                                   earlier blocks.  Batched solves use 1 (their pipelines share the SMs). */
#define BEM_OPT_TC_RESERVE 10   /* SMs the persistent trailing-update kernel (BEM_OPT_TCGEN05 = 2) leaves
                                   to the look-ahead's diagonal and panel kernels (default 0, <= 64) */

/* kernel classes reported by bem_kernel_times */
#define BEM_KC_FAR 0       /* far-field tile kernel of the assembly */
#define BEM_KC_NEAR 1      /* near-singular, on-element and diagonal kernels */
#define BEM_KC_LU_PREP 2   /* equilibration + FP32 copy */
#define BEM_KC_LU_CRIT 3   /* LU critical path: diagonal blocks and panels */
#define BEM_KC_LU_TRAIL 4  /* LU bulk trailing updates (tcgen05) */
#define BEM_KC_TRSV 5      /* triangular solves of the preconditioner */
#define BEM_KC_GEMV 6      /* FP64 matrix-vector products and residuals */
#define BEM_KC_LU_TOTAL 7  /* whole factorization */
#define BEM_KC_LU_DIAG 8   /* diagonal-block factorizations (part of BEM_KC_LU_CRIT) */
#define BEM_KC_LU_PANELS 9 /* panel triangular solves (part of BEM_KC_LU_CRIT) */
#define BEM_KC_LU_THIN 10  /* look-ahead thin updates (own stream) */
#define BEM_KC_COUNT 11

/* solve modes */
#define BEM_SOLVE_FP64 0  /* FP64 assembly + FP64 LU */
#define BEM_SOLVE_MIXED 1 /* FP64 A for the residual, TF32 LU, FP64 GMRES-IR */

/*
 * Boundary mesh of one 2-D problem (the fields `_pack_boundary2d` packs,
 * src/Laplace/Assembly_GPU.jl:169-228, plus the element CAD nodes
 * `Element.geo` and lengths `Element.Length`, src/Core/Structures.jl:317-324).
 * All arrays FP64, host or device memory according to the call's `mem`.
 */
typedef struct bem_geom2d {
  int32_t nt;          /* collocation points (boundary + internal) */
  int32_t n;           /* boundary nodes = ne * (p + 1) */
  int32_t ne;          /* elements */
  int32_t p;           /* field degree: Legendre(p) on Gauss points (1..5) */
  int32_t ngeo;        /* CAD nodes per element (equispaced), 0 = none */
  int32_t reserved;
  const double* px;    /* [nt] collocation x */
  const double* py;    /* [nt] collocation y */
  const double* nx;    /* [n] outward normal x */
  const double* ny;    /* [n] outward normal y */
  const double* jac;   /* [n] |dx/dxi| at each boundary node (Element.Jacobian) */
  const double* elen;  /* [ne] element length (Element.Length) */
  const double* geo_x; /* [ne*ngeo] CAD nodes x (Element.geo), may be NULL if ngeo == 0 */
  const double* geo_y; /* [ne*ngeo] CAD nodes y */
  const double* elem_weight; /* [p+1] Gauss weights of the element rule (dad.elem_weight) */
} bem_geom2d;

typedef struct bem_ctx bem_ctx;

/* Refinement / solve report. */
typedef struct bem_solve_stats {
  int32_t status;        /* BEM_OK or BEM_ERR_NOT_CONVERGED */
  int32_t iterations;    /* GMRES iterations (mixed mode) */
  double rel_residual;   /* ||b - A x|| / ||b|| in FP64 at exit */
  double t_assemble_ms;  /* device time of the assembly */
  double t_factor_ms;    /* device time of the LU */
  double t_refine_ms;    /* device time of the refinement */
  int32_t pivoted;       /* 1: the mixed solve's unpivoted factorization broke down (vanishing
                            pivot) or its refinement stagnated, and the system was solved by LU
                            with partial pivoting in FP64 (BEM_OPT_PIVOT_FALLBACK) */
  int32_t reserved;
} bem_solve_stats;

/* Context: one device, one stream, cached device workspace.  Replaces the
 * per-call KernelAbstractions backend of `_ka_backend`
 * (src/Laplace/Assembly_GPU.jl:152-167). */
int bem_ctx_create(int device, bem_ctx** out);
int bem_ctx_destroy(bem_ctx* ctx);
/* Run subsequent calls on this cudaStream_t (NULL = the context's own). */
int bem_ctx_set_stream(bem_ctx* ctx, void* cuda_stream);
/* Text of the last CUDA error seen by this context. */
const char* bem_last_error(bem_ctx* ctx);
const char* bem_status_string(int status);

/*
 * Dense Laplace H, G.  Replaces `H_G_gpu(dad::BEMdata{<:Laplace}; T, npg,
 * near, near_factor, device, threaded)` (src/Laplace/Assembly_GPU.jl:120-150)
 * and returns what `H_G_full_direct` (src/Core/Assembly_full.jl:61-85)
 * returns: far pairs by nodal lumping, near pairs by the tanp3c map with an
 * npg-point rule, on-element pairs by interpolated Guiggiani, and the
 * row-sum diagonal.  dtype BEM_F32: far entries in FP32 math, near and
 * singular entries in FP64, stored as float; BEM_F64: FP64 throughout.
 * H: ldh >= nt; G: ldg >= nt.
 */
int bem_assemble_laplace2d(bem_ctx* ctx, const bem_geom2d* geom, double k, int npg,
                           double near_factor, int dtype, int mem, void* H, int64_t ldh,
                           void* G, int64_t ldg);

/*
 * Dense Kelvin H, G in 2x2 blocks.  Replaces `H_G_gpu(dad::BEMdata{<:
 * Elasticity}; ...)` (src/Elasticity/Assembly_GPU.jl:15-51) with the values
 * of the vectorial `H_G_full_direct` (src/Core/Assembly_full.jl:120-175).
 * mu: shear modulus; nu_eff: effective Poisson ratio (`effective_nu`,
 * src/Core/Structures.jl:260-263).  H: ldh >= 2nt; G: ldg >= 2nt.
 */
int bem_assemble_kelvin2d(bem_ctx* ctx, const bem_geom2d* geom, double mu, double nu_eff,
                          int npg, double near_factor, int dtype, int mem, void* H, int64_t ldh,
                          void* G, int64_t ldg);

/*
 * Assembly with the boundary-condition column swap fused in: writes the
 * FP64 system A x = b of `applyBC` (src/Core/Boundary_conditions.jl:54-75
 * for Laplace, 152-174 for Kelvin) without forming H and G.  kind 0 =
 * Laplace (prm0 = k), 1 = Kelvin (prm0 = mu, prm1 = nu_eff).  BC/BV have one
 * entry per boundary DOF (0 = primary field prescribed).
 */
int bem_assemble_system2d(bem_ctx* ctx, const bem_geom2d* geom, int kind, double prm0,
                          double prm1, const int32_t* BC, const double* BV, int npg,
                          double near_factor, int mem, double* A, int64_t lda, double* b);

/*
 * Solve a dense FP64 system A x = b (the seam `bem_linsolve(A, b)`,
 * src/Core/LinearSolveUtils.jl:44-49, that `solve` calls,
 * src/Core/Solver.jl:57 and :125).  n x n, column-major, lda >= n.
 *   BEM_SOLVE_MIXED: columns equilibrated, FP32 copy factored by a blocked
 *     LU without pivoting whose updates run on TF32 tensor cores (3xTF32
 *     split), then FP64 restarted GMRES on the FP64 matrix, preconditioned
 *     by that LU, until ||b - A x|| <= tol ||b||, or until a restart cycle no
 *     longer halves a residual below 1e-10 ||b|| (the FP64 rounding floor of
 *     the matrix: x is backward stable, like the reference's LU solution;
 *     stats->rel_residual reports the residual reached), or max_iter
 *     iterations (then BEM_ERR_NOT_CONVERGED with x the last iterate).  A
 *     vanishing pivot of the unpivoted LU, or a refinement that stalls
 *     above that floor, hands the system to LU with partial pivoting in
 *     FP64 (BEM_OPT_PIVOT_FALLBACK, on by default; stats->pivoted = 1).  A is
 *     not modified.
 *   BEM_SOLVE_FP64: LU with partial pivoting in FP64 (cuSOLVER getrf/getrs,
 *     the FP64 comparison path).
 * stats may be NULL.
 */
int bem_solve_system(bem_ctx* ctx, int64_t n, const double* A, int64_t lda, const double* b,
                     int mode, double tol, int max_iter, int mem, double* x,
                     bem_solve_stats* stats);

/*
 * `assemble!` + `solve` in one call: the fused assembly of
 * bem_assemble_system2d followed by bem_solve_system's solve.  x (length
 * dof*nt) is the solution of A x = b; `split_sol!` (src/Core/Solver.jl:88-98,
 * 133-146) maps it to (T, q) or (u, traction) from BC/BV.
 */
int bem_solve2d(bem_ctx* ctx, const bem_geom2d* geom, int kind, double prm0, double prm1,
                const int32_t* BC, const double* BV, int npg, double near_factor, int mode,
                double tol, int max_iter, int mem, double* x, bem_solve_stats* stats);

/* Set a context option (BEM_OPT_*). */
int bem_ctx_set_option(bem_ctx* ctx, int option, int value);

/* Accumulated device time (ms) and launch-group counts per kernel class
 * (BEM_KC_*) since the last call, with BEM_OPT_KERNEL_TIMING on; resets the
 * accumulators.  Tracing facility, no reference counterpart. */
int bem_kernel_times(bem_ctx* ctx, double* ms, int64_t* counts, int n);

/*
 * Timeline of the timed kernel classes (BEM_OPT_KERNEL_TIMING on) since the
 * last call: up to cap records of (class, start ms, end ms), times from the
 * start of the first record of each synchronisation window, in launch order
 * per stream.  Returns the number of records (negative status on error) and
 * clears the timeline.  No reference counterpart (instrumentation).
 */
int bem_kernel_trace(bem_ctx* ctx, int cap, int* cls, double* t0_ms, double* t1_ms);

/* Number of kernel launches made by the library in this process. */
int64_t bem_launch_count(void);

/*
 * Allocation-free Laplace H, G: same results as bem_assemble_laplace2d with
 * BEM_MEM_DEVICE, for callers that cannot allocate device memory while they
 * run (device memory owned by another allocator's pool such as CUDA.jl's or
 * PyTorch's, real-time loops that may only allocate at start-up).  No
 * counterpart in the reference.  It calls no cudaMalloc/cudaFree and needs
 * no bem_ctx: the assembly scratch is a fixed device array of
 * BEM_NOALLOC_BYTES inside the library, present on every GPU that loads the
 * library until the process exits.  Limits: nt <= BEM_NOALLOC_MAX_NT,
 * ne <= BEM_NOALLOC_MAX_NE, at most 24*BEM_NOALLOC_MAX_NT near pairs;
 * larger problems return BEM_ERR_UNSUPPORTED.  The size limits are checked
 * before any device work; the near-pair limit is only known after the
 * assembly ran, so when it is exceeded the call returns BEM_ERR_UNSUPPORTED
 * with H and G written but undefined (the pairs beyond the limit keep far-field
 * values).  The element weights are read on cuda_stream, after the caller's
 * earlier work on it.  geom, H and G are device
 * pointers; work runs on cuda_stream (NULL = legacy default stream) and the
 * call returns when it is done.  The first call on each device looks up the
 * array's address (loading the module) and should precede any stream
 * capture.  All calls share the one array: calls that overlap on the GPU
 * race, so callers must serialize them.
 */
#define BEM_NOALLOC_MAX_NT 16384
#define BEM_NOALLOC_MAX_NE 8192
#define BEM_NOALLOC_BYTES 4456704
int bem_assemble_laplace2d_noalloc(const bem_geom2d* geom, double k, int npg, double near_factor,
                                   int dtype, void* H, int64_t ldh, void* G, int64_t ldg,
                                   void* cuda_stream);

/*
 * Dense pairwise DIBEM matrices over the nt collocation points (x, y):
 * F_ij = phi(R) and D_ij = fundamental solution, i != j, R = |x_j - x_i| --
 * replaces `_dibem_FD_ka` / `_dibem_FD_kernel!` (src/Laplace/DIBEM_GPU.jl:179-208,
 * kind 0 Laplace, prm0 = k, D nt x nt) and `_elast_dibem_FD_kernel!`
 * (src/Elasticity/Assembly_GPU.jl:258-280, kind 1 Kelvin, prm0 = mu, prm1 =
 * effective nu, D 2nt x 2nt of 2x2 U blocks).  rbf: 1-7 polyharmonic
 * splines, 10 fundamental solution (`_gpu_rbf_kind`, DIBEM_GPU.jl:103-114);
 * epsa: the log shift (`AVOID_INF` = 1e-16 in the reference).  dtype BEM_F32
 * computes and stores FP32, BEM_F64 FP64.  F, D column-major.
 */
int bem_dibem_fd2d(bem_ctx* ctx, int nt, const double* px, const double* py, int kind, double prm0, double prm1,
                   int rbf, double epsa, int dtype, int mem, void* F, int64_t ldf, void* D, int64_t ldd);

/*
 * Far boundary sums of the DIBEM domain integrals over the collocation
 * points of a 2-D Laplace mesh -- replaces `_dibem_IFID_ka` /
 * `_dibem_IFID_kernel!` (src/Laplace/DIBEM_GPU.jl:209-270): for each point i,
 *   IF_i = sum_j phi_int(R) w_j (r . n_j) / R^2,  ID_i = sum_j rad(R) w_j (r . n_j) / R^2
 * over boundary nodes j with R = |x_j - x_i| > 1e-10, skipping the element
 * of j when it is near x_i (near_factor, the assembly's exact test) or holds
 * x_i (`_near_skip_mask`, src/Laplace/Assembly_GPU.jl:236-253); phi_int and
 * rad are `_dibem_phi_int2d` / `_dibem_rad_id2d` (DIBEM_GPU.jl:141-177),
 * w_j = Jacobian_j elem_weight_k.  The near-pair quadrature correction stays
 * with the caller, as in the reference.  rbf as in bem_dibem_fd2d; dtype
 * BEM_F32 / BEM_F64 the arithmetic and output type; IF, ID [nt].
 */
int bem_dibem_ifid2d(bem_ctx* ctx, const bem_geom2d* geom, double k, int rbf, double epsa, double near_factor,
                     int dtype, int mem, void* IF, void* ID);

/*
 * Boundary discretisation: ne elements, each given by ngeo equispaced CAD
 * nodes (cad_x/cad_y [ne*ngeo], element-major), to p+1 collocation nodes per
 * element at the Gauss-Legendre points with the Jacobian |dx/dxi|, the
 * outward normal (tangent rotated by -90 degrees) and the element length
 * |sum_k J_k w_k| -- the geometry loop of `format2d`
 * (src/Core/Input.jl:163-185) and `bemdata_from_loops`
 * (src/Topology/Topology.jl:311-319).  Outputs px, py, nx, ny, jac [ne*(p+1)]
 * and elen [ne] fill a bem_geom2d directly; elem_weight (host, [p+1]) gets
 * the Gauss weights.  mem says where cad_* and the outputs live (elem_weight
 * is always host).  2 <= ngeo <= 6, 0 <= p <= 5.
 */
int bem_discretize2d(bem_ctx* ctx, int ne, int ngeo, int p, const double* cad_x, const double* cad_y, int mem,
                     double* px, double* py, double* nx, double* ny, double* jac, double* elen,
                     double* elem_weight);

/*
 * Near-pair correction of the DIBEM boundary sums -- replaces
 * `_dibem_correct_near_cpu!` (src/Laplace/DIBEM_GPU.jl:272-300), which the
 * reference runs on the host after `_dibem_IFID_ka`: adds to IF, ID (FP64,
 * [nt], in and out) the npg-point Gauss-rule integrals of every element near
 * a point (the assembly's near test, near_factor) or holding it, on the
 * element's field interpolant (`_rim_build_elements`,
 * src/Core/DIBEM_common.jl:112-171).  With bem_dibem_ifid2d (whose far sums
 * skip exactly those pairs) it gives the reference's IF, ID.  rbf as in
 * bem_dibem_fd2d; mem says where IF, ID live (geometry as in the other calls).
 */
int bem_dibem_ifid_near2d(bem_ctx* ctx, const bem_geom2d* geom, double k, int rbf, double epsa,
                          double near_factor, int npg, int mem, double* IF, double* ID);

/*
 * Outward normals of a 2-D boundary mesh -- replaces `_orient_normals_outward!`
 * (src/Core/Input.jl:376-389) of `format2d`: for element e (nodes e(p+1) ..
 * e(p+1)+p of px, py, nx, ny; length elen[e]) the point 0.1 elen[e] behind
 * its first node along -n must lie inside one of the ncell domain cells (the
 * 2-D elements of the mesh, even-odd test of `point_in_polygon`, :331-345),
 * else all of the element's normals are negated in place; flipped[e] = 1
 * then.  cells: ncell x 4 corners (x, y), a triangle repeating its last
 * corner.  ncell = 0 leaves the normals unchanged, as the reference does
 * without a 2-D mesh.  mem says where all arrays live.
 */
int bem_orient2d(bem_ctx* ctx, int ne, int p, const double* px, const double* py, double* nx, double* ny,
                 const double* elen, int ncell, const double* cells, int mem, int32_t* flipped);

/*
 * Shape gradient by the adjoint method (no reference counterpart; built on
 * the path's assembly and solve, src/Core/Assembly_full.jl:61-175 and
 * src/Core/Boundary_conditions.jl:20-75).  Laplace, elements with their
 * geometry from their own nodes (geom->ngeo = 0), no internal points.
 * J = 1/2 sum over nodes with BC = 0 of (q_i - q_target_i)^2, with q from the
 * mixed-precision solve; grad receives dJ/dx_j, dJ/dy_j (2n, node-major)
 * with BC, BV and q_target held fixed.  The influence entries are
 * recomputed in the backward kernels, not stored.  mem says where BC, BV,
 * q_target, J and grad live (geometry as in the other calls).
 */
int bem_adjoint_laplace2d(bem_ctx* ctx, const bem_geom2d* geom, double k, const int32_t* BC, const double* BV,
                          const double* q_target, int npg, double near_factor, double tol, int max_iter,
                          int mem, double* J, double* grad, bem_solve_stats* stats);

/*
 * Batched solves of ndom independent domains with uneven sizes (the
 * reference solves one mesh per `solve(dad)` call, src/Core/Solver.jl:24-64;
 * there is no batched counterpart).  Domain d is geoms[d]; its BC/BV entries
 * start at BC + bc_off[d], BV + bc_off[d] (dof * n_d of them) and its solution
 * is written to x + x_off[d] (dof * nt_d values).  Every domain runs the
 * bem_solve2d pipeline (same arguments for all); nworkers host threads, each
 * with its own stream and workspace, take domains largest first (0 = 8,
 * at most 32).  stats (optional) receives one record per domain.  Returns
 * the first error met, BEM_ERR_NOT_CONVERGED if a domain stopped short of
 * tol, else BEM_OK.  The call is synchronous.
 */
int bem_solve2d_batch(bem_ctx* ctx, int ndom, const bem_geom2d* geoms, int kind, double prm0, double prm1,
                      const int32_t* BC, const double* BV, const int64_t* bc_off, int npg, double near_factor,
                      int mode, double tol, int max_iter, int mem, double* x, const int64_t* x_off,
                      int nworkers, bem_solve_stats* stats);

/*
 * bem_adjoint_laplace2d for ndom independent domains on nworkers worker
 * streams (0 = 8, at most 32), largest domains first; host buffers only.
 * Domain d's BC, BV and q_target entries start at offset off[d] (n_d of
 * each), its gradient at grad + 2 off[d] (2 n_d values) and its misfit is
 * J[d].  stats (optional) receives one record per domain.  Returns as
 * bem_solve2d_batch.  The call is synchronous.
 */
int bem_adjoint_laplace2d_batch(bem_ctx* ctx, int ndom, const bem_geom2d* geoms, double k, const int32_t* BC,
                                const double* BV, const double* q_target, const int64_t* off, int npg,
                                double near_factor, double tol, int max_iter, double* J, double* grad,
                                int nworkers, bem_solve_stats* stats);

/*
 * Laplace potential at m interior points from solved boundary data --
 * replaces `interior_laplace(dad, pf; T, q)` (src/Laplace/Lubrication.jl:399-416;
 * the same sum as `_interior_T`, test/laplace.jl:36-53): every element is
 * integrated with the near-field quadrature of `integrate_element`
 * (src/Core/Assembly_full.jl:262-289), T(p) = (g.q - h.T) / c, c = -sum h.
 * T, q: the n boundary values (`dad.T[1:n]`, `dad.q`); xp, yp: point
 * coordinates; out: m potentials.  mem says where T, q, xp, yp, out live.
 */
int bem_interior_laplace2d(bem_ctx* ctx, const bem_geom2d* geom, double k, int npg, const double* T,
                           const double* q, int64_t m, const double* xp, const double* yp, int mem,
                           double* out);

/*
 * Boundary strain and stress at the n collocation nodes of a solved Kelvin
 * problem (Kane's method) -- replaces `recover_strain_stress!`
 * (src/Elasticity/StrainStress.jl:35-53, 2-D branch `_recover_2d!`, :55-99).
 * lam, mu: Lame constants of the effective 2-D model (`props.lambda`,
 * `props.mu`, src/Core/Structures.jl:160-168).  u, t: node-major
 * displacement and traction (2n each, `dad.u`, `dad.traction`).  eps, sigma:
 * n x 3 column-major Voigt (e11, e22, g12) and (s11, s22, s12), as the
 * reference's `zeros(n, 3)`.  mem says where u, t, eps and sigma live.
 */
int bem_strain_stress2d(bem_ctx* ctx, const bem_geom2d* geom, double lam, double mu, const double* u,
                        const double* t, int mem, double* eps, double* sigma);

/*
 * Built-in consistency check of the tensor-core paths (no reference
 * counterpart).  which = 1: factor an n x n test matrix (n a multiple of 128)
 * once with the tcgen05 trailing updates and once with the legacy mma.sync
 * updates; out[0] = max |difference of the factors|, out[1] = max |factor|,
 * out[2], out[3] = factorization times in ms (tcgen05, legacy).  which = 2:
 * the 128 x 128 diagonal-block factorization against a reference kernel.
 * which = 3: the bulk trailing update of one LU step, C ((n-128)^2) -= L U,
 * timed alone: out[0] ms per launch, out[1] algorithmic GB/s (C read and
 * write), out[2] TF32 tensor TFLOP/s (three products).  n >= 256.
 * which = 4 (BEM_OPT_TCGEN05 = 2): the persistent and the per-tile bulk
 * update on the same operands, over the whole trailing matrix and over its
 * part past the first block row and column; out[0], out[1] = max |difference|,
 * max |entry| of the first shape, out[2], out[3] the same for the second.
 */
int bem_selftest(bem_ctx* ctx, int which, int n, double* out);

#ifdef __cplusplus
}
#endif
#endif /* BEM_GB300_H */
