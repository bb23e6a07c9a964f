#!/usr/bin/env python3
"""Headline benchmark: dense 2-D Laplace BEM solve at N = 8193 on one GB300.

Workload (the N=8192 configuration, restated as seeded synthetic geometry):
star-shaped boundary r(t) = 1 + sum_{k=2..6} a_k cos(k t + phi_k), a_k ~
U(0, 0.08), phi_k ~ U(0, 2 pi) (seed 0), 2731 discontinuous quadratic
elements (N = 8193: 8192 is not a multiple of 3 nodes per element), field
T = e^x cos y with Dirichlet data where the element starts at t in [0, pi)
and Neumann data on [pi, 2 pi), npg = 16 near-field rule.

One step = one solve: fused assembly of A x = b (far field, near-singular
and singular integrals, boundary-condition swap) + FP32 tensor-core LU +
FP64 GMRES refinement to ||b - A x|| <= 1e-14 ||b||.  `value` is solves/s
with the geometry and boundary data already resident on the device; `e2e`
is the same through the public host-buffer API (host->device copy of the
inputs and device->host copy of x inside each step).  The FP64 comparison
path (FP64 assembly + cuSOLVER LU) is timed on the same input.

--impl reference times the CPU restatement of the reference's own path
(assembly on all host threads + LAPACK LU), the CPU implementation of this
path, on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
# the batched solve drives up to 32 worker streams, each with side streams:
# 32 hardware work queues instead of the default 8 keep them from sharing
# queues (set before the first CUDA call of the process)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

METRIC = ("solves/sec & H+G entries/sec at N=8192, mixed vs FP64 GPU, "
          "≤1e-10 rel err vs FP64")
def workload(ne, npg):
    return (f"star-shaped Laplace domain, {ne} quadratic elements, N={3 * ne} collocation nodes, "
            f"npg={npg}, mixed Dirichlet/Neumann data for T=exp(x)cos(y), seed 0")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 50 ms in the background."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def reduce_max(x, device):
    """Max of x over the ranks of the default process group (x itself on one
    process): the slowest replica sets the whole job's time."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_reference(dad_factory, steps, warmup, npg):
    """The CPU restatement of the path: oracle assembly (all host threads) +
    applyBC + LAPACK LU (SciPy/OpenBLAS, all threads)."""
    from oracle import oracle as orc
    ts = []
    x = None
    stages = {}
    for it in range(warmup + steps):
        dad = dad_factory()
        r = orc.timed_pipeline(dad, npg=npg, threads=os.cpu_count() or 1)
        if it >= warmup:
            ts.append(r["total"])
        x = r["x"]
        stages = {k: r[k] for k in ("assemble", "apply_bc", "lu")}
    return ts, x, stages


# DRAM traffic of one bulk trailing update (k_gemm_tc_p, the persistent
# kernel) at the C2 trailing size, from one ncu capture of the update timed
# alone (bem_selftest which = 3, n = 8192, trailing block 8064^2):
# dram__bytes_read 276934400 B + dram__bytes_write 200425984 B for
# 8 * 8064^2 = 520224768 algorithmic bytes.
GEMM_TRAFFIC_CAPTURE = {"launch": "bulk update alone, trailing block 8064^2", "read_bytes": 276934400,
                        "write_bytes": 200425984, "algorithmic_bytes": 8 * 8064 ** 2}


def extra_configs(ctx):
    """Config C4 (512 uneven star domains, batched solve), C3 (plate with a
    hole, 8196 DOF elasticity) and C5 (adjoint shape gradients of 64 domains
    x 1023 nodes), wall-clock through the public API with host buffers."""
    import numpy as np
    from bem_gmsh_gb300.geometry import c4_node_counts, c4_domains, star_adjoint_case
    from bem_gmsh_gb300.api import solve_batch, adjoint_laplace, adjoint_laplace_batch, solve, tune_batch
    out = {}
    sizes = c4_node_counts(512, seed=0)
    dads = c4_domains(sizes)
    # warm-up: the autotuner's passes (one at 32 workers, then one per
    # candidate count) size every worker's workspace, so that the timed pass
    # allocates nothing, and choose the worker count it runs with
    workers, tuning = tune_batch(dads, npg=16, mode="mixed", candidates=(8, 16, 24, 32), ctx=ctx)
    t = time.perf_counter()
    xs, st = solve_batch(dads, npg=16, mode="mixed", nworkers=0, ctx=ctx, return_stats=True)
    dt = time.perf_counter() - t
    ent = float(np.sum(sizes.astype(float) ** 2))
    idx = np.linspace(0, len(dads) - 1, 64).astype(int)
    sub = [c4_domains([sizes[i]], seed0=100 + int(i))[0] for i in idx]  # same domains, fresh copies
    t64 = time.perf_counter()
    xf = solve_batch(sub, npg=16, mode="fp64", nworkers=16, ctx=ctx)
    dt64 = time.perf_counter() - t64
    errs = [float(np.linalg.norm(xs[i] - f) / np.linalg.norm(f)) for i, f in zip(idx, xf)]
    out["batched_c4"] = {
        "domains": len(dads), "nodes_min": int(sizes.min()), "nodes_max": int(sizes.max()),
        "sum_entries": ent, "seconds": dt, "solves_per_s": len(dads) / dt, "entries_per_s": ent / dt,
        "workers": workers, "tuning_s": {str(k): round(v, 4) for k, v in tuning.items()},
        "max_gmres_iterations": int(max(s["iterations"] for s in st)),
        "fp64_sample": {"domains": len(idx), "seconds": dt64, "max_rel_err": max(errs),
                        "median_rel_err": float(np.median(errs))},
        "note": "wall clock through solve_batch with host buffers, after the autotuner's passes; "
                "per-domain pipelines on the tuned number of worker streams"}
    # C3: plate with a hole, 8196 DOF of 2-D elasticity, mixed vs FP64 GPU
    from bem_gmsh_gb300.geometry import plate_with_hole
    from bem_gmsh_gb300.api import recover_strain_stress, hoop_stress
    s_inf = 1e8
    plate = plate_with_hole(n_outer_el=1024, n_hole_el=342, p=2, sigma=s_inf)
    for _ in range(2):
        solve(plate, npg=16, mode="mixed", ctx=ctx)
    tm, stm = [], []
    for _ in range(10):
        t0 = time.perf_counter()
        _, stc = solve(plate, npg=16, mode="mixed", ctx=ctx, return_stats=True)
        tm.append(time.perf_counter() - t0)
        stm.append(stc)
    x3 = plate.cache["x"].copy()
    recover_strain_stress(plate, ctx=ctx)
    hole = np.arange(plate.n - 3 * 342, plate.n)
    Xh = np.asarray(plate.collocation[hole])
    th = np.arctan2(Xh[:, 1], Xh[:, 0])
    stt = hoop_stress(plate)[hole] / s_inf
    top = np.abs(np.abs(th) - np.pi / 2) < 0.02
    p64 = plate_with_hole(n_outer_el=1024, n_hole_el=342, p=2, sigma=s_inf)
    solve(p64, npg=16, mode="fp64", ctx=ctx)
    t64 = []
    for _ in range(2):
        t0 = time.perf_counter()
        solve(p64, npg=16, mode="fp64", ctx=ctx)
        t64.append(time.perf_counter() - t0)
    x64 = p64.cache["x"]
    free = np.asarray(plate.BC) == 1
    nt3, n3 = plate.nt, plate.n
    ent3 = float((2 * nt3) * (2 * nt3) + (2 * nt3) * (2 * n3))
    asm_ms = statistics.mean(sv["t_assemble_ms"] for sv in stm)
    out["plate_c3"] = {
        "dof": 2 * nt3, "solves_per_s": 1.0 / statistics.mean(tm), "ms_per_solve": 1e3 * statistics.mean(tm),
        "fp64_solves_per_s": 1.0 / statistics.mean(t64),
        "speedup_mixed_vs_fp64": statistics.mean(t64) / statistics.mean(tm),
        "rel_err_displacements_vs_fp64_gpu": float(np.linalg.norm(x3[free] - x64[free]) /
                                                   np.linalg.norm(x64[free])),
        "pinned_reactions_diff_over_load": float(np.max(np.abs(x3[~free] - x64[~free])) / s_inf),
        "assembly_ms": asm_ms, "entries_per_s": ent3 / (asm_ms * 1e-3),
        "factor_ms": statistics.mean(sv["t_factor_ms"] for sv in stm),
        "refine_ms": statistics.mean(sv["t_refine_ms"] for sv in stm),
        "gmres_iterations": int(max(sv["iterations"] for sv in stm)),
        "kirsch_peak_hoop_stress": float(stt[top].mean()),
        "note": "wall clock of api.solve with host buffers (10 mixed, 2 FP64 solves); mixed: Kelvin far "
                "field in double-float, FP32/TF32 LU, FP64 GMRES; stage times are device time; H+G entries "
                "(2nt)^2 + (2nt)(2n) per assembly; errors of the displacement unknowns (relative) and of the "
                "three pinned reaction tractions (zero for this self-equilibrated load, relative to the "
                "load); the hoop-stress peak at the top and bottom of the hole (3.879 in a converged oracle "
                "mesh study); the full-size comparison with the FP64 oracle is tests/test_gpu_stress.py"}
    cases = [star_adjoint_case(341, p=2, seed=s) for s in range(64)]
    qts = []
    for d, tg in cases:
        solve(tg, npg=16, mode="mixed", ctx=ctx)
        qts.append(np.where(tg.BC == 0, tg.cache["x"], 0.0))
    adjoint_laplace(cases[0][0], qts[0], npg=16, ctx=ctx)
    t = time.perf_counter()
    res = [adjoint_laplace(d, q, npg=16, ctx=ctx, return_stats=True) for (d, _), q in zip(cases, qts)]
    dt_seq = time.perf_counter() - t
    # the same 64 gradients through the batched entry point (one warm-up pass
    # sizes the workers' workspaces)
    pairs = [(d, q) for (d, _), q in zip(cases, qts)]
    adjoint_laplace_batch(pairs, npg=16, nworkers=16, ctx=ctx)
    t = time.perf_counter()
    resb, stb = adjoint_laplace_batch(pairs, npg=16, nworkers=16, ctx=ctx, return_stats=True)
    dt = time.perf_counter() - t
    gdiff = max(float(np.linalg.norm(gb - r[1]) / np.linalg.norm(r[1])) for (_, gb), r in zip(resb, res))
    # DIBEM pairwise F, D over the C2 points (device buffers, kernel time)
    import torch
    from bem_gmsh_gb300 import _lib as L
    from bem_gmsh_gb300.geometry import star_domain
    d2 = star_domain(2731, p=2, seed=0)
    nt = d2.nt
    pts = torch.as_tensor(np.asarray(d2.collocation, np.float64)).cuda()
    px, py = pts[:, 0].contiguous(), pts[:, 1].contiguous()
    hbm_gbs = peaks()[0]
    dib = {}
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    for name, tdt, dtid in (("fp32", torch.float32, L.BEM_F32), ("fp64", torch.float64, L.BEM_F64)):
        ldx = (nt + 3) // 4 * 4
        Fb = torch.empty((nt, ldx), dtype=tdt, device="cuda")
        Db = torch.empty((nt, ldx), dtype=tdt, device="cuda")

        def run():
            rc = ctx.L.bem_dibem_fd2d(ctx.h, nt, px.data_ptr(), py.data_ptr(), 0, 1.0, 0.0, 3, 1e-16, dtid,
                                      L.BEM_MEM_DEVICE, Fb.data_ptr(), ldx, Db.data_ptr(), ldx)
            ctx.check(rc, "dibem_fd")
        for _ in range(3):
            run()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(10)]
        for e0, e1 in ev:
            e0.record(stream)
            run()
            e1.record(stream)
        torch.cuda.synchronize()
        ms = sum(e0.elapsed_time(e1) for e0, e1 in ev) / len(ev)
        nbytes = 2.0 * nt * nt * Fb.element_size()
        dib[name] = {"ms": ms, "entries_per_s": 2.0 * nt * nt / (ms * 1e-3),
                     "hbm_frac": nbytes / (ms * 1e-3) / 1e9 / hbm_gbs}
        del Fb, Db
    ctx.set_stream(0)
    # DIBEM far boundary sums IF, ID at the C2 points (nt x n pairs)
    from bem_gmsh_gb300.api import dibem_ifid
    for name, tdt in (("ifid_fp32", np.float32), ("ifid_fp64", np.float64)):
        dibem_ifid(d2, rbf="PHS3", dtype=tdt, ctx=ctx)
        t0 = time.perf_counter()
        for _ in range(5):
            dibem_ifid(d2, rbf="PHS3", dtype=tdt, ctx=ctx)
        ms = (time.perf_counter() - t0) / 5 * 1e3
        dib[name] = {"ms": ms, "pairs_per_s": float(nt) * d2.n / (ms * 1e-3),
                     "note": "wall clock per call through the API with host buffers"}
    out["dibem_fd_c2"] = {"N": nt, "rbf": "PHS3", **dib,
                          "note": "F and D (2 N^2 entries) written to device buffers; CUDA events on the "
                                  "launching stream around each call (one launch, plus its launch latency)"}
    out["adjoint_c5"] = {
        "domains": len(cases), "nodes": cases[0][0].n, "seconds": dt, "gradients_per_s": len(cases) / dt,
        "ms_per_gradient": 1e3 * dt / len(cases), "workers": 16,
        "sequential_ms_per_gradient": 1e3 * dt_seq / len(cases),
        "max_rel_diff_batch_vs_sequential": gdiff,
        "max_iterations_fwd_plus_adj": int(max(s["iterations"] for s in stb)),
        "note": "J and dJ/d(node x, y): forward + adjoint mixed solves and the backward kernels, 64 domains "
                "through adjoint_laplace_batch (wall clock, host buffers); finite-difference checks against "
                "the FP64 oracle are in tests/test_gpu_adjoint.py"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ne", type=int, default=2731)
    ap.add_argument("--npg", type=int, default=16)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=0, help="end-to-end solves timed (0: the same as --steps)")
    ap.add_argument("--cpu-samples", type=int, default=1)
    ap.add_argument("--no-extra", action="store_true", help="skip the batched (C4) and adjoint (C5) lines")
    args = ap.parse_args()
    assert args.warmup >= 3 or args.impl == "reference" or args.warmup >= 0

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    from bem_gmsh_gb300.geometry import star_domain, rel_error

    def make():
        return star_domain(args.ne, p=2, seed=0)

    if args.impl == "reference":
        if rank != 0:
            return
        ts, _, _ = cpu_reference(make, max(1, args.steps), min(args.warmup, 1), args.npg)
        v = 1.0 / statistics.mean(ts)
        cores = os.cpu_count() or 1
        line = {"metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus, "steps": len(ts),
                "warmup": min(args.warmup, 1), "ms_per_step": 1e3 * statistics.mean(ts),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "impl": "reference",
                "config": {"workload": workload(args.ne, args.npg), "N": 3 * args.ne, "npg": args.npg},
                "cpu_baseline": {"value": v, "unit": "solves/s", "cores": cores, "kind": "port",
                                 "sample": f"{len(ts)} full solves of the workload (assembly on {cores} "
                                           f"threads + LAPACK LU)"},
                "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import numpy as np
    import torch

    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    from bem_gmsh_gb300 import _lib
    from bem_gmsh_gb300.api import geom_struct, solve, split_sol

    ctx = _lib.default_context(local_rank if world > 1 else 0)
    dad = make()
    N = dad.nt
    # device-resident inputs
    g, keep = geom_struct(dad, device=True)
    BC = torch.as_tensor(np.asarray(dad.BC, np.int32)).cuda()
    BV = torch.as_tensor(np.asarray(dad.BV, np.float64)).cuda()
    x = torch.zeros(N, dtype=torch.float64, device="cuda")
    st = _lib.BemSolveStats()

    def step(mode):
        rc = ctx.L.bem_solve2d(ctx.h, g, 0, float(dad.properties.k), 0.0, BC.data_ptr(), BV.data_ptr(),
                               args.npg, 1.5, mode, 1e-14, 200, _lib.BEM_MEM_DEVICE, x.data_ptr(), st)
        ctx.check(rc, "bem_solve2d")

    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    for _ in range(args.warmup):
        step(_lib.BEM_SOLVE_MIXED)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    l0 = ctx.launch_count()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    iters = []
    for _ in range(args.steps):
        step(_lib.BEM_SOLVE_MIXED)
        iters.append(st.iterations)
    e1.record(stream)
    torch.cuda.synchronize()
    launches = ctx.launch_count() - l0
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    # kernel classes: a separate pass with the library's per-class CUDA events
    # on (kept out of the timed loop above)
    prof_steps = min(args.steps, 10)
    ctx.set_option(_lib.BEM_OPT_KERNEL_TIMING, 1)
    ctx.kernel_times()
    for _ in range(prof_steps):
        step(_lib.BEM_SOLVE_MIXED)
    torch.cuda.synchronize()
    ktimes = ctx.kernel_times()
    ctx.set_option(_lib.BEM_OPT_KERNEL_TIMING, 0)
    ms = reduce_max(ms, "cuda")
    value = world * 1e3 / ms
    x_mixed = x.cpu().numpy().copy()
    stats_mixed = dict(iterations=st.iterations, rel_residual=st.rel_residual,
                       t_assemble_ms=st.t_assemble_ms, t_factor_ms=st.t_factor_ms, t_refine_ms=st.t_refine_ms)

    # FP64 comparison path
    step(_lib.BEM_SOLVE_FP64)  # warm-up (library load, workspace)
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(args.fp64_steps):
        step(_lib.BEM_SOLVE_FP64)
    f1.record(stream)
    torch.cuda.synchronize()
    ms64 = f0.elapsed_time(f1) / args.fp64_steps
    x64 = x.cpu().numpy().copy()
    rel_vs_fp64 = float(np.linalg.norm(x_mixed - x64) / np.linalg.norm(x64))

    # assembly throughput: H and G in FP32 (device resident)
    ld = (N + 3) // 4 * 4
    Hs = torch.empty((N, ld), dtype=torch.float32, device="cuda")
    Gs = torch.empty((dad.n, ld), dtype=torch.float32, device="cuda")
    H = Hs.t()[:N]
    G = Gs.t()[:N]

    def asm():
        rc = ctx.L.bem_assemble_laplace2d(ctx.h, g, 1.0, args.npg, 1.5, _lib.BEM_F32, _lib.BEM_MEM_DEVICE,
                                          H.data_ptr(), ld, G.data_ptr(), ld)
        ctx.check(rc, "assemble")
    for _ in range(3):
        asm()
    torch.cuda.synchronize()
    a0 = torch.cuda.Event(enable_timing=True)
    a1 = torch.cuda.Event(enable_timing=True)
    a0.record(stream)
    for _ in range(args.steps):
        asm()
    a1.record(stream)
    torch.cuda.synchronize()
    ms_asm = a0.elapsed_time(a1) / args.steps
    entries = N * N + N * dad.n
    entries_per_s = entries / (ms_asm * 1e-3)
    del Hs, Gs
    # the same H, G in FP64 (the FP64 comparison path's assembly)
    Hd = torch.empty((N, ld), dtype=torch.float64, device="cuda")
    Gd = torch.empty((dad.n, ld), dtype=torch.float64, device="cuda")

    def asm64():
        rc = ctx.L.bem_assemble_laplace2d(ctx.h, g, 1.0, args.npg, 1.5, _lib.BEM_F64, _lib.BEM_MEM_DEVICE,
                                          Hd.t()[:N].data_ptr(), ld, Gd.t()[:N].data_ptr(), ld)
        ctx.check(rc, "assemble fp64")
    asm64()
    torch.cuda.synchronize()
    a0.record(stream)
    n64 = max(1, min(args.steps, 5))
    for _ in range(n64):
        asm64()
    a1.record(stream)
    torch.cuda.synchronize()
    ms_asm64 = a0.elapsed_time(a1) / n64
    del Hd, Gd

    # end to end through the public API (host buffers)
    ctx.set_stream(0)
    e2e_dad = make()
    solve(e2e_dad, npg=args.npg, mode="mixed", ctx=ctx)
    te = []
    e2e_steps = args.e2e_steps or args.steps
    for _ in range(e2e_steps):
        t0 = time.perf_counter()
        solve(e2e_dad, npg=args.npg, mode="mixed", ctx=ctx)
        te.append(time.perf_counter() - t0)
    e2e_ms = 1e3 * statistics.mean(te)
    h2d = sum(a.nbytes for a in (e2e_dad.collocation, e2e_dad.normal, e2e_dad.jacobian, e2e_dad.elem_length,
                                 e2e_dad.geo, e2e_dad.elem_weight, e2e_dad.BC, e2e_dad.BV))
    d2h = 8 * N

    # roofline of every kernel class over the timed region, and of the dominant one.
    # achieved = algorithmic units of one solve x steps / device time of the class.
    hbm, bf16, src = peaks()
    nb = (N + 127) // 128 * 128
    rems = [nb - (k + 1) * 128 for k in range(nb // 128)]
    iters_last = max(1, iters[-1] if iters else 1)
    algo = {
        # bytes: the FP64 system matrix A written once
        "far": ("hbm", 8.0 * N * N, "GB/s", "FP64 A written, 8 B/entry"),
        # bytes: 8 B/pair of listed near pairs is negligible; FP64 issue bound
        "near": ("hbm", 8.0 * 24 * N, "GB/s", "near/singular entries, FP64 issue bound"),
        # bytes: FP64 A read twice (column scales, conversion) + FP32 copy written
        "lu_prep": ("hbm", 16.0 * N * N + 4.0 * nb * nb, "GB/s", "A64 read x2 + A32 written"),
        # flops: diagonal block (4/3 128^3) + both panels (4 128^2 rem) + the
        # look-ahead column and row block updates (4 128^2 rem) per step
        "lu_crit": ("tensor", sum(4.0 / 3.0 * 128 ** 3 + 8.0 * 128 * 128 * r for r in rems), "TFLOP/s",
                    "latency-bound chain: one diagonal block per step on one SM"),
        # bytes: the bulk trailing update reads and writes its FP32 block once
        # per step, 8 rem'^2 B (3xTF32 intensity 96 flop/B is below the TF32
        # machine balance, so HBM bounds it); operands come from L2
        "lu_trail": ("hbm", sum(8.0 * max(r - 128, 0) ** 2 for r in rems), "GB/s",
                     "tcgen05 3xTF32 trailing updates (k_gemm_tc_p): C read + write per step"),
        # bytes: FP32 L and U read once per preconditioner application
        "trsv": ("hbm", 4.0 * nb * nb * iters_last, "GB/s", "FP32 LU read per sweep pair"),
        # bytes: one FP64 A read per product (one per iteration + the final
        # residual; the first residual from x = 0 is b itself)
        "gemv": ("hbm", 8.0 * N * N * (iters_last + 1), "GB/s", "FP64 A read per product"),
    }
    classes = {}
    for k, (bound, units, unit, note) in algo.items():
        ms_k = ktimes.get(k, (0.0, 0))[0]
        if ms_k <= 0:
            continue
        ach = units * prof_steps / (ms_k * 1e-3) / (1e9 if bound == "hbm" else 1e12)
        pk = hbm if bound == "hbm" else bf16
        classes[k] = {"bound": bound, "achieved": ach, "unit": unit, "peak": pk, "frac": ach / pk,
                      "ms_per_step": ms_k / prof_steps, "note": note}
    # the dominant kernel of the ncu launch list is the tcgen05 GEMM
    # of the bulk trailing update; its class is lu_trail
    dom = "lu_trail" if "lu_trail" in classes else max(classes, key=lambda k: classes[k]["ms_per_step"])
    roof = dict(classes[dom])
    flops_trail = sum(2.0 * max(r - 128, 0) ** 2 * 128 for r in rems)
    cap = GEMM_TRAFFIC_CAPTURE
    ratio = (cap["read_bytes"] + cap["write_bytes"]) / cap["algorithmic_bytes"]
    nbulk = max(1, sum(1 for r in rems if r > 128))
    roof.update({"kernel": "k_gemm_tc_p (persistent bulk trailing update)", "kernel_class": dom,
                 "traffic": ratio * algo["lu_trail"][1] / nbulk,
                 "traffic_note": "bytes per average bulk launch: the measured DRAM read+write / algorithmic "
                                 "ratio of one full-size ncu capture (%s, %.3f) times the algorithmic bytes "
                                 "of the average launch; writes still in L2 at kernel end are not counted"
                                 % (cap["launch"], ratio),
                 "peak_source": src,
                 "peak_note": "measured copy bandwidth",
                 "tensor_view": {"algorithmic_tflops": flops_trail * prof_steps / (ktimes["lu_trail"][0] * 1e-3) / 1e12,
                                 "tf32_mma_tflops": 3 * flops_trail * prof_steps / (ktimes["lu_trail"][0] * 1e-3) / 1e12,
                                 "tf32_dense_peak_tflops": bf16 / 2}})

    # replicas: the e2e time is the slowest rank's too
    e2e_ms = reduce_max(e2e_ms, "cuda")

    extra = {}
    if not args.no_extra and world == 1:
        extra = extra_configs(ctx)

    # CPU baseline (N = 1 only): the oracle port on the host cores, one full
    # solve sample
    cpu_fields = {}
    if world == 1:
        cpu_ts, x_orc, cpu_stages = cpu_reference(make, max(1, args.cpu_samples), 0, args.npg)
        cores = os.cpu_count() or 1
        cpu_v = 1.0 / statistics.mean(cpu_ts)
        cpu_fields = {
            "rel_err_vs_cpu_oracle": float(np.linalg.norm(x_mixed - x_orc) / np.linalg.norm(x_orc)),
            "rel_error_analytic_cpu": None,
            "cpu_stages": {"assembly_ms": 1e3 * cpu_stages["assemble"],
                           "entries_per_s": (N * N + N * dad.n) / cpu_stages["assemble"],
                           "apply_bc_ms": 1e3 * cpu_stages["apply_bc"], "lu_ms": 1e3 * cpu_stages["lu"],
                           "note": "oracle assembly on all host threads, LAPACK LU"},
            "cpu_baseline": {"value": cpu_v, "unit": "solves/s", "cores": cores, "kind": "port",
                             "sample": f"{len(cpu_ts)} full solve(s) of the same workload: oracle assembly on "
                                       f"{cores} threads + LAPACK LU"},
        }

    def analytic_error(x):
        d = make()
        split_sol(d, x)
        return float(rel_error(d))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32/tf32+fp64-ir", "data": "synthetic",
            "config": {"workload": workload(args.ne, args.npg), "N": N, "npg": args.npg, "mode": "mixed (FP32/TF32 LU + FP64 GMRES)",
                       "tol": 1e-14, "l2": "inputs larger than L2 (FP64 system 537 MB)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "entries_per_s": entries_per_s, "assembly_ms_fp32_HG": ms_asm,
            "fp64_solves_per_s": 1e3 / ms64, "fp64_ms_per_step": ms64,
            "speedup_mixed_vs_fp64": ms64 / ms,
            "rel_err_vs_fp64_gpu": rel_vs_fp64,
            "rel_error_analytic": float(rel_error(e2e_dad)),
            "rel_error_analytic_fp64_gpu": analytic_error(x64),
            "fp64_assembly_ms_HG": ms_asm64, "fp64_entries_per_s": entries / (ms_asm64 * 1e-3),
            "gmres_iterations": iters[-1] if iters else None, "stats": stats_mixed,
            "kernel_ms_per_step": {k: v[0] / prof_steps for k, v in ktimes.items()},
            "e2e": {"value": world * 1e3 / e2e_ms, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": e2e_steps,
                    "note": "mean wall clock of api.solve with host buffers (host-to-device copies of the "
                            "geometry and boundary data, device-to-host copy of the solution)"},
            "roofline": roof, "roofline_classes": classes,
            "clocks": clk, "gpu_launches": int(launches),
        }
        if cpu_fields:
            cpu_fields["rel_error_analytic_cpu"] = analytic_error(x_orc)
        line.update(cpu_fields)
        line.update(extra)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
