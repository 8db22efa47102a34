"""Benchmark: sshex8 Laplacian matrix-free apply at L=4 on a 48^3 macro mesh, and solves.

Workload (one "step"): one FP32 apply y += A x of the affine sshex8 Laplacian
(level 4, 48x48x48 macro hex8 elements of the unit cube, interior macro nodes
perturbed by U(-0.1,0.1) h, seed 0): 110,592 macro elements, 7,189,057 nodes.
FP32 is the precision the mixed-precision solvers apply the operator in.
``value`` = GDoF/s with x, y and the mesh resident in HBM; the L2 cache is
flushed (a 512 MiB write, then a 512 MiB read that retires the write's dirty lines)
before every timed step and kernels are timed with
CUDA events on the launching stream.  ``e2e`` = the same apply through the C
ABI with host buffers: every step copies x from pinned host memory, zeroes y,
applies and copies y back to pinned host memory; consecutive steps overlap on
three streams (copy in, compute, copy out; double-buffered).
``fp64_apply`` = the FP64 apply (the precision of the oracle parity, 1e-13).
``solve`` = time to a true FP64 relative residual, plain FP64 multigrid-CG
against the mixed-precision solvers (Poisson 48^3 L=4, elasticity cantilever
64x16x16 L=4), and the batched serving run (256 uneven problems).

``--impl reference`` times the reference's CPU algorithm for the same apply in the
same precision: the oracle's restatement of affine_sshex8_laplacian_stencil_apply_fff
(the reference's default CPU path: 27-point stencil inside each macro element, partial
stencils on its surface) in the reference's float32 number configuration, OpenMP on
every host core the process may use, OMP_PROC_BIND=true.  The restatement is pinned to
the reference's own build of that function (FP64 and float32 configurations) by the
CPU test suite.
"""

from __future__ import annotations

import argparse
import json
import os

# host threads this process may use, read before any OpenMP runtime starts (with
# OMP_PROC_BIND the runtime pins the calling thread to one core afterwards)
try:
    HOST_CORES = len(os.sched_getaffinity(0))
except AttributeError:
    HOST_CORES = os.cpu_count()
# thread binding of the OpenMP CPU baseline, as the reference's run scripts set it;
# before any import that starts an OpenMP runtime
os.environ.setdefault("OMP_PROC_BIND", "true")
os.environ.setdefault("OMP_NUM_THREADS", str(HOST_CORES))
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

NX = 48
LEVEL = 4
METRIC = "sshex8 Laplacian apply GDoF/s (FP32, L=4, 48^3 macro); solve times to FP64 residual in 'solve'"
NOMINAL_FP64_TFLOPS = 1.25  # GB300 nominal FP64 (no measured figure in the peaks file)
# dram__bytes_read.sum + dram__bytes_write.sum of one launch of the step's kernel (the FP32
# node-centric stencil kernel on packed tiles) on this workload, from an ncu capture of
# `bench.py --profile-apply` (cold cache, mean of two launches: 115.51 MB read + 5.32 MB
# written)
TRAFFIC_BYTES_PER_LAUNCH = 120.83e6
SEED = 0
PERTURB = 0.1


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=NX)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--profile-kernels", action="store_true",
                    help="launch each main kernel twice on the bench workloads and exit (an ncu target)")
    ap.add_argument("--profile-apply", action="store_true",
                    help="launch only the 48^3 L=4 Laplacian applies (FP32 stencil and element-matrix kernels, "
                         "FP64 stencil kernel) twice each and exit (an ncu target)")
    ap.add_argument("--batch-problems", type=int, default=256)
    ap.add_argument("--profile-zoo", action="store_true",
                    help="launch every vector, SpMV and coarse-level kernel twice on inputs larger than L2 "
                         "(a target for per-kernel ncu captures)")
    ap.add_argument("--profile-solves", action="store_true",
                    help="run one mixed + learned Poisson solve (32^3 L=4, k = exp(g)) and one mixed elasticity "
                         "solve (64x16x16 L=4) (a target for solver launch-list captures)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_config(nx):
    from sfem_gb300.mesh import SSMesh

    m = SSMesh(nx, nx, nx, LEVEL, perturb=PERTURB, seed=SEED)
    return m


L2_NOTE = ("flushed before every timed step, after the y reset: 512 MiB write, then 512 MiB read of another "
           "buffer (the write's dirty lines leave L2 before the timed region)")


def config_dict(m, world=1):
    """The workload description both arms print (identical keys and values; `l2` is the
    GPU arm's timing rule, the CPU arm's caches are described in its cpu_baseline)."""
    return {"workload": "sshex8_laplacian_apply_L4_48cube", "nodes": m.n_nodes(), "macro_elements": m.n_elements,
            "level": LEVEL, "perturb": PERTURB, "seed": SEED, "l2": L2_NOTE,
            "parallelism": f"replicas{world}" if world > 1 else "single"}


def stencil_fma_per_element(L):
    """FMAs of the node-centric apply per macro element: 27 taps inside, 18 on faces,
    12 on edges, 8 at corners (2,197 at L = 4)."""
    return 27 * (L - 1) ** 3 + 18 * 6 * (L - 1) ** 2 + 12 * 12 * (L - 1) + 8 * 8


def host_cores():
    """Host threads the CPU baseline runs on: the process's affinity mask at start-up
    (OMP_NUM_THREADS is set to it)."""
    return int(os.environ.get("OMP_NUM_THREADS", HOST_CORES))


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._thr = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits"],
                    capture_output=True, text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([s.strip() for s in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._thr = threading.Thread(target=self._run, daemon=True)
        self._thr.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._thr:
            self._thr.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 3 + k and "Active" in s[3 + k]
                          and "Not" not in s[3 + k]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def replica_aggregate(t_local: float, units_per_rank: float, world: int, device=None):
    """Whole-job throughput of independent replicas: every rank processes the same
    units; the job time is the max over ranks (all_reduce MAX when world > 1)."""
    t = float(t_local)
    if world > 1:
        import torch
        import torch.distributed as dist

        tt = torch.tensor([t], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    return world * units_per_rank / t, t


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def cpu_apply_time(m, dtype, reps=3):
    """Seconds per apply of the oracle's restatement of the reference's CPU stencil apply
    (OpenMP, every host core of the affinity mask) on the full mesh."""
    import oracle as O

    el = m.elements(LEVEL)
    fff = O.fff_fill(el[m.macro_corner_lidx(LEVEL)], m.points)
    x = np.random.default_rng(1).standard_normal(m.n_nodes())
    if dtype == "f32":
        x = x.astype(np.float32)
        fn = lambda out: O.sshex8_laplacian_stencil_apply_f32(LEVEL, el, fff, x, out=out)
    else:
        fn = lambda out: O.sshex8_laplacian_stencil_apply(LEVEL, el, fff, x, out=out)
    y = np.zeros_like(x)
    fn(y)  # warm-up
    t = time.perf_counter()
    for _ in range(reps):
        y[:] = 0
        fn(y)
    return (time.perf_counter() - t) / reps


CPU_KIND_NOTE = ("oracle restatement of affine_sshex8_laplacian_stencil_apply_fff "
                 "(operators/sshex8/sshex8_laplacian.cpp:698-769; stencil form), float32 number configuration, "
                 "OpenMP, OMP_PROC_BIND=true; pinned to the reference's own float32 build of that function")


def cpu_baseline(m, reps=3):
    """The reference's CPU stencil apply (oracle restatement, float32 configuration) on the host cores."""
    dt = cpu_apply_time(m, "f32", reps)
    return {"value": m.n_nodes() / dt / 1e9, "unit": "GDoF/s", "cores": host_cores(), "kind": "port",
            "sample": f"{reps} FP32 applies of the full 48^3 L=4 mesh, after one warm-up apply",
            "algorithm": CPU_KIND_NOTE, "omp_proc_bind": os.environ.get("OMP_PROC_BIND"),
            "seconds_per_apply": dt}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    m = workload_config(args.nx)
    import oracle as O

    el = m.elements(LEVEL)
    fff = O.fff_fill(el[m.macro_corner_lidx(LEVEL)], m.points)
    x = np.random.default_rng(1).standard_normal(m.n_nodes()).astype(np.float32)
    y = np.zeros_like(x)
    for _ in range(max(1, args.warmup)):
        O.sshex8_laplacian_stencil_apply_f32(LEVEL, el, fff, x, out=y)
    steps = max(1, min(args.steps, 20))  # bounded CPU sample
    t = time.perf_counter()
    for _ in range(steps):
        y[:] = 0
        O.sshex8_laplacian_stencil_apply_f32(LEVEL, el, fff, x, out=y)
    dt = (time.perf_counter() - t) / steps
    v = m.n_nodes() / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": v,
        "unit": "GDoF/s", "n_gpus": world, "steps": steps, "warmup": args.warmup, "ms_per_step": dt * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_dict(m, world),
        "cpu_baseline": {"value": v, "unit": "GDoF/s", "cores": host_cores(), "kind": "port",
                         "sample": f"{steps} timed FP32 applies of the full 48^3 L=4 mesh",
                         "algorithm": CPU_KIND_NOTE, "omp_proc_bind": os.environ.get("OMP_PROC_BIND"),
                         "caches": "not flushed; one apply's data (~144 MB) exceeds the host caches"},
        "e2e": {"value": v, "unit": "GDoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def measure_e2e(op, x, N, steps, world, dev):
    """GDoF/s of the streamed apply through the C ABI with host buffers (see run_ours)."""
    import ctypes

    import torch

    xh = torch.empty(N, dtype=torch.float32, pin_memory=True)
    xh.copy_(x.cpu())
    yh = [torch.empty(N, dtype=torch.float32, pin_memory=True) for _ in range(2)]
    xd = [torch.empty_like(x) for _ in range(2)]
    yd = [torch.empty_like(x) for _ in range(2)]
    s_in, s_cmp, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    h_cmp = ctypes.c_void_p(s_cmp.cuda_stream)
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_cmp = [torch.cuda.Event() for _ in range(2)]
    ev_out = [torch.cuda.Event() for _ in range(2)]

    def step(k):
        b = k % 2
        with torch.cuda.stream(s_in):
            s_in.wait_event(ev_cmp[b])  # step k - 2's apply has read xd[b]
            xd[b].copy_(xh, non_blocking=True)
            ev_in[b].record(s_in)
        with torch.cuda.stream(s_cmp):
            s_cmp.wait_event(ev_in[b])
            s_cmp.wait_event(ev_out[b])  # step k - 2's result has left yd[b]
            yd[b].zero_()
            op.apply(xd[b], yd[b], stream=ctypes.byref(h_cmp))
            ev_cmp[b].record(s_cmp)
        with torch.cuda.stream(s_out):
            s_out.wait_event(ev_cmp[b])
            yh[b].copy_(yd[b], non_blocking=True)
            ev_out[b].record(s_out)

    for k in range(4):
        step(k)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(s_in)
    for k in range(steps):
        step(k)
    s_out.wait_stream(s_in)
    s_out.wait_stream(s_cmp)
    e1.record(s_out)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / steps
    return world * N / t / 1e9, t


class L2Flush:
    """Evicts the L2 before a timed step: a 512 MiB write (no input of the step stays
    cached), then a 512 MiB read of another buffer, so the dirty lines of the write are
    written back before the timed region instead of competing with the step's traffic."""

    def __init__(self, dev):
        import torch

        self.w = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)
        self.r = torch.zeros(64 * 1024 * 1024, dtype=torch.float64, device=dev)

    def __call__(self, k):
        self.w.fill_(k & 0xFF)
        self.r.sum()


def time_apply(op, x, y, steps, warmup, flush, stream):
    """Mean CUDA-event time of op.apply(x, y) with the L2 flushed before every step."""
    import torch

    for _ in range(max(3, warmup)):
        y.zero_()
        op.apply(x, y)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        y.zero_()
        flush(k)  # after the reset, so y too comes from HBM
        starts[k].record(stream)
        op.apply(x, y)
        ends[k].record(stream)
    torch.cuda.synchronize()
    return float(np.mean([a.elapsed_time(b) for a, b in zip(starts, ends)])) / 1e3


def _timed_solve(S, solver, b, x):
    import torch

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rc = S.solve(solver, b, x)
    torch.cuda.synchronize()
    return rc, time.perf_counter() - t0


def refine_dd(S, res, inner, b, x, rtol, max_outer=8, x_lo=None, stall=0.5):
    """Iterative refinement driven by the compensated residual: r = b - A x in
    double-double (``res``), stop when ||r|| / ||b|| <= rtol, else solve A e = r with
    the inner solver from e = 0 and update x += e -- in FP64, or error-free into the
    double-double solution (x, x_lo) when x_lo is given.  ``inner`` may be a list: step
    k uses inner[min(k, len - 1)].  Also stops when a step fails to cut the residual by
    the factor ``stall`` (the floor of an FP64 solution vector).  Returns (relative
    residual, outer steps, inner iterations, stalled)."""
    inners = inner if isinstance(inner, (list, tuple)) else [inner]
    import torch

    nb = torch.linalg.vector_norm(b)
    e = torch.zeros_like(b)
    r = res(x, b, x_lo=x_lo)
    rel = float(torch.linalg.vector_norm(r) / nb)
    outer = inner_its = 0
    stalled = False
    while rel > rtol and outer < max_outer:
        inner = inners[min(outer, len(inners) - 1)]
        e.zero_()
        S.solve(inner, r, e)
        inner_its += S.stats(inner)[0]
        if x_lo is None:
            x += e
        else:
            S.dd_axpy(1.0, e, x, x_lo)
        res(x, b, r, x_lo=x_lo)
        new = float(torch.linalg.vector_norm(r) / nb)
        outer += 1
        stalled = new > stall * rel
        rel = new
        if stalled:
            break
    return rel, outer, inner_its, stalled


def _timed(fn):
    import torch

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def oracle_residuals_laplacian(m, fff_aos, dn, x, b):
    """FP64 and double-double residuals of a GPU solution evaluated by the oracle on the host."""
    import oracle as O

    el = m.elements(LEVEL)
    Ax = O.sshex8_laplacian_stencil_apply(LEVEL, el, fff_aos, x)
    Ax[dn] = x[dn]
    rd = O.laplacian_residual_dd(LEVEL, el, fff_aos, x, b)
    rd[dn] = b[dn] - x[dn]
    nb = np.linalg.norm(b)
    return {"fp64": float(np.linalg.norm(b - Ax) / nb), "double_double": float(np.linalg.norm(rd) / nb)}


def oracle_residuals_elasticity(m, adj_aos, det, mu, lam, dn, x, b):
    import oracle as O

    el = m.elements(LEVEL)
    Kx = O.linear_elasticity_apply(LEVEL, el, adj_aos, det, mu, lam, x)
    rd = O.elasticity_residual_dd(LEVEL, el, adj_aos, det, mu, lam, x, b)
    for c in range(3):
        Kx[3 * dn + c] = x[3 * dn + c]
        rd[3 * dn + c] = b[3 * dn + c] - x[3 * dn + c]
    nb = np.linalg.norm(b)
    return {"fp64": float(np.linalg.norm(b - Kx) / nb), "double_double": float(np.linalg.norm(rd) / nb)}


def measure_solves(m, dev, rtol=1e-10, cpu_solve=True):
    """Time to ||b - A x|| / ||b|| <= rtol on the Poisson problem of the 48^3 L=4 mesh,
    same hierarchy for every arm (sshex8 levels 4, 2, 1, then hex8 levels coarsening the
    macro grid; Jacobi-scaled Chebyshev3 V(2,2); dense coarsest solve; V-cycles replayed
    as CUDA graphs):
      plain: FP64 flexible CG + FP64 multigrid;
      mixed_ir: FP64 iterative refinement around FP32 CG + FP32 multigrid;
      mixed_precond: FP64 flexible CG preconditioned by the FP32 multigrid (FP64 only for
      the residual, dot products and solution update).
    Every arm's residual is certified after the solve by the compensated (double-double)
    GPU residual and by the oracle on the host (FP64 and double-double); the solutions are
    compared with the oracle's CPU multigrid-CG solution (the CPU solve baseline)."""
    import torch

    import oracle as O
    from sfem_gb300 import solvers as S

    H = S.Hierarchy(m, dirichlet_faces=("x0",), device=dev, coarsen_macro=True)
    N = m.n_nodes()
    g = torch.Generator(device=dev).manual_seed(SEED + 7)
    b = torch.randn(N, dtype=torch.float64, device=dev, generator=g)
    b[H.dirichlet[0].long()] = 0
    ctx = S.context()
    op64 = S.laplacian_op(ctx, H.spaces[0], H.fff, H.dirichlet[0], torch.float64)
    res = S.CompensatedResidual(H, "laplacian")
    out = {"levels_nodes": [sp.n_nodes for sp in H.spaces], "rtol": rtol,
           "smoother": "Jacobi-scaled Chebyshev3 V(2,2)", "coarse": "dense Cholesky inverse on the coarsest hex8 level",
           "vcycle": "CUDA graph replay", "fine_operator": "node-centric stencil kernel (FP64 and FP32)"}

    def true_rel(x):
        r = torch.zeros_like(b)
        S.apply(op64, x, r)
        return float(torch.linalg.vector_norm(b - r) / torch.linalg.vector_norm(b))

    t0 = time.perf_counter()
    mg64, _ = S.build_poisson_mg(ctx, H, torch.float64, smoother="chebyshev3", sweeps=2, coarse="dense", graph=True)
    torch.cuda.synchronize()
    setup64 = time.perf_counter() - t0
    cg64 = S.cg(ctx, op64, mg64, rtol=rtol, max_it=500, residual_norm=True, flexible=True)
    x = torch.zeros_like(b)
    rc, t64 = _timed_solve(S, cg64, b, x)
    sols = {"plain_fp64_mg_pcg": x}
    out["plain_fp64_mg_pcg"] = {"seconds": t64, "iterations": S.stats(cg64)[0], "true_rel_residual": true_rel(x),
                                "rc": rc, "setup_seconds": setup64}
    x64 = x.clone()
    xn = float(torch.linalg.vector_norm(x64))
    t0 = time.perf_counter()
    mg32, op32 = S.build_poisson_mg(ctx, H, torch.float32, smoother="chebyshev3", sweeps=2, eig_max=mg64.eigs,
                                    coarse="dense", graph=True)
    torch.cuda.synchronize()
    setup32 = time.perf_counter() - t0
    inner = S.cg(ctx, op32, mg32, rtol=1e-4, max_it=30, residual_norm=True, flexible=True)
    ir = S.iterative_refinement(ctx, op64, inner, max_it=30, rtol=rtol)
    x = torch.zeros_like(b)
    rc, tir = _timed_solve(S, ir, b, x)
    sols["mixed_ir"] = x
    out["mixed_ir"] = {"seconds": tir, "outer_iterations": S.stats(ir)[0], "true_rel_residual": true_rel(x),
                       "rc": rc, "setup_seconds": setup32,
                       "solution_rel_diff_vs_plain_fp64": float(torch.linalg.vector_norm(x - x64)) / xn}
    pc = S.mixed_precond(ctx, mg32)
    cgm = S.cg(ctx, op64, pc, rtol=rtol, max_it=500, residual_norm=True, flexible=True)
    x = torch.zeros_like(b)
    rc, tpc = _timed_solve(S, cgm, b, x)
    sols["mixed_precond"] = x
    out["mixed_precond"] = {"seconds": tpc, "iterations": S.stats(cgm)[0], "true_rel_residual": true_rel(x),
                            "rc": rc, "solution_rel_diff_vs_plain_fp64": float(torch.linalg.vector_norm(x - x64)) / xn}
    ok = all(out[a]["rc"] == 0 and out[a]["true_rel_residual"] <= rtol for a in sols)
    out["speedup_mixed_ir_vs_plain"] = t64 / tir if ok else None
    out["speedup_mixed_precond_vs_plain"] = t64 / tpc if ok else None
    # certification: compensated GPU residual, and the oracle on the host
    fff_aos = H.fff.cpu().numpy().T.copy()
    dn = H.dirichlet[0].long().cpu().numpy()
    bh = b.cpu().numpy()
    for a, xs in sols.items():
        out[a]["double_double_rel_residual"] = res.relative(xs, b)
        out[a]["oracle_rel_residual"] = oracle_residuals_laplacian(m, fff_aos, dn, xs.cpu().numpy(), bh)
    if cpu_solve:
        out["cpu_solve"] = cpu_solve_laplacian(m, fff_aos, bh, {a: xs.cpu().numpy() for a, xs in sols.items()}, rtol)
    return out


def cpu_solve_laplacian(m, fff_aos, b, gpu_solutions, rtol):
    """The oracle's CPU multigrid-CG (restated reference CG + V-cycle + Chebyshev3, OpenMP
    on every host core) on the same problem: its time to the true residual rtol, and
    the GPU solutions' distance to its solution."""
    import oracle as O

    x, st = O.mg_pcg_solve(m, "laplacian", b, geom=fff_aos, sweeps=2, scaled=True, scale_eig_max=1.02,
                           coarse_rtol=1e-8, rtol=rtol, max_it=100, flexible=True)
    xn = np.linalg.norm(x)
    st.update({"cores": host_cores(), "kind": "port",
               "algorithm": "oracle/src/solve.c: flexible CG + V(2,2) multigrid on the sshex8 levels 4, 2, 1, "
                            "Jacobi-scaled Chebyshev3 (power-method eigenvalue x 1.02), Jacobi-CG coarse solve to "
                            "rtol 1e-8 on the macro hex8 level (the reference's mgsolve settings), stencil-form "
                            "FP64 applies",
               "gpu_solution_rel_diff": {a: float(np.linalg.norm(xs - x) / xn) for a, xs in gpu_solutions.items()}})
    return st


def lumped_body_force(m, det):
    """Lumped-mass load of a unit body force in -z: node i gets sum over micro elements
    containing it of |micro element| / 8 (affine sub-elements: |e| = det_macro / L^3)."""
    L = m.L
    el = m.elements(L)
    N1 = L + 1
    lid = np.arange(N1 ** 3)
    xi, yi, zi = lid % N1, (lid // N1) % N1, lid // (N1 * N1)
    mult = np.ones(N1 ** 3)
    for c in (xi, yi, zi):
        mult *= np.where((c == 0) | (c == L), 1.0, 2.0)  # micro elements of this macro element sharing the node
    w = (mult[:, None] * (det.astype(np.float64) / (8.0 * L ** 3))[None, :])
    vol = np.bincount(el.reshape(-1), weights=w.reshape(-1), minlength=m.n_nodes())
    b = np.zeros(3 * m.n_nodes())
    b[2::3] = -vol
    return b


def measure_elasticity_solves(dev, nx=64, ny=16, nz=16, rtol=1e-10, mu=1.0, lam=10.0, inner_rtol=(1e-6, 3e-5),
                               cpu_solve=False):
    """Cantilever 4x1x1, macro 64x16x16 at L=4, clamped at x=0, lumped body force (0,0,-1).
    Both arms are driven to a relative residual of rtol by iterative refinement on the
    compensated (double-double) GPU residual, each refinement step solving A e = r to
    inner_rtol with
      plain: FP64 flexible CG + FP64 multigrid;
      mixed_precond: FP64 flexible CG preconditioned by the FP32 multigrid (FP32
      operator on the tcgen05 3xTF32 kernel at L=4).
    Same hierarchy, smoother, dense coarsest solve and graph-replayed V-cycles for both.
    The clamped 4:1 cantilever has |A||x| / |b| near 1e6, which puts the plain-FP64
    evaluation of the residual near 1e-10: the compensated residual is what certifies
    rtol, and the oracle re-evaluates every solution on the host in FP64 and in
    double-double."""
    import torch

    from sfem_gb300 import solvers as S
    from sfem_gb300.mesh import SSMesh

    m = SSMesh(nx, ny, nz, LEVEL, box=((0, 4), (0, 1), (0, 1)), perturb=0.0, seed=SEED)
    H = S.Hierarchy(m, dirichlet_faces=("x0",), device=dev, vec=3, coarsen_macro=True)
    b = torch.from_numpy(lumped_body_force(m, H.det.cpu().numpy())).to(dev)
    for c in range(3):
        b[3 * H.dirichlet[0].long() + c] = 0
    ctx = S.context()
    op64 = S.elasticity_op(ctx, H.spaces[0], H.adj, H.det, mu, lam, H.dirichlet[0], torch.float64)
    res = S.CompensatedResidual(H, "elasticity", mu=mu, lam=lam)

    def fp64_rel(x):
        r = torch.zeros_like(b)
        S.apply(op64, x, r)
        return float(torch.linalg.vector_norm(b - r) / torch.linalg.vector_norm(b))

    out = {"dofs": 3 * m.n_nodes(), "macro_elements": m.n_elements, "levels_nodes": [sp.n_nodes for sp in H.spaces],
           "rtol": rtol, "inner_rtol": list(inner_rtol), "smoother": "Jacobi-scaled Chebyshev3 V(2,2)",
           "coarse": "dense Cholesky inverse on the coarsest hex8 level", "vcycle": "CUDA graph replay",
           "outer": "iterative refinement on the compensated (double-double) residual"}
    mg64, _ = S.build_elasticity_mg(ctx, H, torch.float64, mu=mu, lam=lam, coarse="dense", graph=True)
    mg32, _ = S.build_elasticity_mg(ctx, H, torch.float32, mu=mu, lam=lam, eig_max=mg64.eigs, coarse="dense",
                                    graph=True)
    # refinement step k solves to inner_rtol[k] (the last one repeats): a first solve to
    # 1e-6, then a correction that needs only the remaining factor
    pc32 = S.mixed_precond(ctx, mg32)
    arms = {"plain_fp64_mg_pcg": [S.cg(ctx, op64, mg64, rtol=t, max_it=500, residual_norm=True, flexible=True)
                                  for t in inner_rtol],
            "mixed_precond": [S.cg(ctx, op64, pc32, rtol=t, max_it=500, residual_norm=True, flexible=True)
                              for t in inner_rtol]}
    sols = {}
    for name, inner in arms.items():
        for k in range(len(inner)):  # warm-up: capture every graph once
            refine_dd(S, res, inner[k:], b, torch.zeros_like(b), rtol, max_outer=1)
        # the solution kept in double-double (x, x_lo): the refinement reaches rtol
        x, xl = torch.zeros_like(b), torch.zeros_like(b)
        (rel, outer, its, _), sec = _timed(lambda: refine_dd(S, res, inner, b, x, rtol, x_lo=xl))
        sols[name] = x
        # the same refinement with a plain FP64 solution vector: it stops at the floor that
        # rounding the solution to FP64 leaves (measured, both residual evaluations)
        x64v = torch.zeros_like(b)
        (rel64, outer64, its64, stalled), sec64 = _timed(lambda: refine_dd(S, res, inner, b, x64v, rtol))
        out[name] = {"seconds": sec, "outer_steps": outer, "iterations": its, "double_double_rel_residual": rel,
                     "rc": int(rel > rtol), "solution": "double-double (x_hi + x_lo)",
                     "rounded_solution_rel_residual": {"double_double": res.relative(x, b),
                                                       "fp64_evaluation": fp64_rel(x)},
                     "fp64_solution_vector": {"seconds": sec64, "outer_steps": outer64, "iterations": its64,
                                              "double_double_rel_residual": rel64, "stalled": stalled,
                                              "fp64_evaluation_rel_residual": fp64_rel(x64v)}}
    x64 = sols["plain_fp64_mg_pcg"]
    out["mixed_precond"]["solution_rel_diff_vs_plain_fp64"] = float(
        torch.linalg.vector_norm(sols["mixed_precond"] - x64) / torch.linalg.vector_norm(x64))
    ok = all(out[a]["rc"] == 0 for a in arms)
    out["speedup_mixed_precond_vs_plain"] = (out["plain_fp64_mg_pcg"]["seconds"] / out["mixed_precond"]["seconds"]
                                             if ok else None)
    if not ok:
        out["speedup_note"] = "an arm missed rtol: no speed-up reported"
    adj_aos = H.adj.cpu().numpy().T.copy()
    det = H.det.cpu().numpy()
    dn = H.dirichlet[0].long().cpu().numpy()
    bh = b.cpu().numpy()
    for a, xs in sols.items():
        out[a]["oracle_rel_residual"] = oracle_residuals_elasticity(m, adj_aos, det, mu, lam, dn, xs.cpu().numpy(), bh)
    if cpu_solve:
        import oracle as O

        x, st = O.mg_pcg_solve(m, "elasticity", bh, geom=adj_aos, det=det, mu=mu, lam=lam, sweeps=2, scaled=True,
                               scale_eig_max=1.1, coarse_rtol=1e-6, rtol=rtol, max_it=400, flexible=True)
        xn = np.linalg.norm(x)
        st.update({"cores": host_cores(), "kind": "port",
                   "gpu_solution_rel_diff": {a: float(np.linalg.norm(xs.cpu().numpy() - x) / xn)
                                             for a, xs in sols.items()}})
        out["cpu_solve"] = st
    return out


def measure_learned(dev, nx=32, draws=64, n_pairs=100_000, epochs=20, eval_draws=2):
    """Config 4: sshex8 L=4 on a 32^3 macro mesh, k = exp(g) per macro element (GRF,
    sigma 1, correlation length 8 macro elements), N(0,1) rhs.  The 3-layer BF16 conv
    smoother is trained by the project's kernels on 10^5 residual/error pairs from plain
    V-cycles on 64 coefficient draws, then every arm solves fresh draws to FP64 1e-10
    with flexible CG: FP64 multigrid (plain), + learned correction, FP32 multigrid
    through the precision bridge (mixed), + learned correction (mixed_learned).  Plain
    and mixed smooth with Chebyshev3 V(2,2); in the learned arms the post-smoothing is
    the learned correction followed by one Chebyshev3 sweep (the correction takes the
    place of the second sweep)."""
    from sfem_gb300 import learned

    res = learned.run_experiment(nx=nx, draws=draws, n_pairs=n_pairs, epochs=epochs, eval_draws=eval_draws,
                                 device=str(dev), placement="before", fallback_sweeps=1)
    arms = list(res["eval"][0].keys())
    out = {"nx": nx, "draws": draws, "pairs": res["pairs"], "epochs": epochs, "placement": res["placement"],
           "smoothing": {"plain_and_mixed": "Chebyshev3 V(2,2)",
                         "learned_arms": "pre: 2 Chebyshev3 sweeps; post: learned correction + 1 Chebyshev3 sweep"},
           "loss_first": res["loss_first"], "loss_last": res["loss_last"], "harvest_seconds": res["harvest_seconds"],
           "train_seconds": res["train_seconds"]}
    for a in arms:
        rows = [r[a] for r in res["eval"]]
        out[a] = {"seconds": float(np.mean([r["seconds"] for r in rows])),
                  "iterations": [r["iterations"] for r in rows],
                  "true_rel_residual_max": max(r["true_rel_residual"] for r in rows),
                  "rc": max(r["rc"] for r in rows), "fallback_used": any(r["fallback_used"] for r in rows)}
    base = out["chebyshev3"]["seconds"]
    for a in arms:
        out[f"speedup_{a}_vs_plain_fp64"] = base / out[a]["seconds"]
    return out


def measure_batch(dev, count=256, seed=0):
    """Batched serving: ``count`` uneven Poisson / elasticity problems (cube edge 8..32
    macro elements, L in {2, 3, 4}, perturbation 0.1 h, N(0,1) rhs, seeded) solved
    together to FP64 relative residual 1e-10 (batched FP64 flexible CG, FP32 multigrid
    per group, chunks of 5 iterations replayed as one CUDA graph); launch shape from
    the autotuner.  Latency of a problem = time from the start of the batch solve
    until the host saw it converged."""
    import torch

    from sfem_gb300.batch import BatchSolver, draw_problems

    t0 = time.perf_counter()
    probs = draw_problems(count, seed=seed)
    bs = BatchSolver(probs, device=dev)
    b = bs.rhs()
    torch.cuda.synchronize()
    setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    table = bs.autotune(b)
    tune = time.perf_counter() - t0
    x = torch.zeros_like(b)
    rc, lat, its, sec = bs.solve(b, x)
    tr = bs.true_residuals(b, x)
    kinds = [p.kind for p in bs.problems]
    out = {
        "problems": count, "dofs": int(bs.n), "groups": len(bs.groups), "rc": int(rc), "seconds": sec,
        "solves_per_s": count / sec,
        "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
        "iterations_max": int(its.max()), "max_true_rel_residual": float(tr.max()),
        "all_converged": bool(rc == 0 and (tr <= 1.5e-10).all()),
        "poisson": kinds.count("poisson"), "elasticity": kinds.count("elasticity"),
        "setup_seconds": setup, "autotune_seconds": tune,
        "autotune": [{"chunk": c[0], "threads": c[1], "ctas_per_sm": c[2], "kernels": k, "ms_per_chunk": t}
                     for c, k, t in table],
        "autotune_kernels": "laplacian: -1 per-level default, 0 staged 64-element tiles, 2 thread per element, "
                            "8 stencil tiles; elasticity: -1 tcgen05 at L=4, 0 SIMT",
        "tuned": list(bs.tuned), "tuned_kernels": bs.tuned_kernels,
    }
    # staggered arrivals: Poisson process over the first half of the simultaneous solve's
    # time, in a seeded random order; latency from each problem's own release
    rng = np.random.default_rng(seed + 1)
    gaps = rng.exponential(1.0, count)
    release = np.cumsum(gaps) / gaps.sum() * 0.5 * sec
    release = release[rng.permutation(count)] - release.min()
    x = torch.zeros_like(b)
    rc2, lat2, its2, sec2 = bs.solve(b, x, release=release)
    tr2 = bs.true_residuals(b, x)
    out["staggered"] = {
        "arrivals": "Poisson process over [0, 0.5 x the simultaneous solve time], seeded, random order",
        "last_release_s": float(release.max()), "rc": int(rc2), "seconds": sec2, "solves_per_s": count / sec2,
        "latency_from_release_p50_s": float(np.percentile(lat2, 50)),
        "latency_from_release_p99_s": float(np.percentile(lat2, 99)),
        "max_true_rel_residual": float(tr2.max()), "all_converged": bool(rc2 == 0 and (tr2 <= 1.5e-10).all()),
    }
    tuned, tuned_kernels = bs.tuned, bs.tuned_kernels
    del bs, b, x
    torch.cuda.empty_cache()
    out["concurrent_groups"] = measure_batch_concurrent(dev, probs, tuned, tuned_kernels)
    torch.cuda.empty_cache()
    out["sequential_gpu"] = measure_batch_sequential(dev, probs, stride=8)
    return out


def measure_batch_concurrent(dev, probs, launch, kernels):
    """The same 256 problems, one batched solver per group on its own stream, each group
    stepping as soon as its last convergence mask arrives (all submitted at t = 0)."""
    import torch

    from sfem_gb300.batch import ConcurrentBatchSolver

    t0 = time.perf_counter()
    cs = ConcurrentBatchSolver(probs, device=dev, launch=launch, kernels=kernels)
    bs = cs.rhs()
    xs = [torch.zeros_like(b) for b in bs]
    torch.cuda.synchronize()
    setup = time.perf_counter() - t0
    lat, its, sec = cs.solve(bs, xs)
    tr = cs.true_residuals(bs, xs)
    res = {
        "groups": len(cs.subs), "stream_priority": "smaller groups on higher-priority streams (6 levels)",
        "seconds": sec, "solves_per_s": len(probs) / sec,
        "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
        "iterations_max": int(its.max()), "max_true_rel_residual": float(tr.max()),
        "all_converged": bool((tr <= 1.5e-10).all()), "setup_seconds": setup,
    }
    del cs, bs, xs
    return res


def measure_batch_sequential(dev, probs, stride=8):
    """The same mixed solver run one problem at a time (a batch of one: FP64 flexible CG,
    FP32 multigrid, graph-replayed chunks) on every ``stride``-th problem of the batched
    draw; solve time only (setup excluded, as for the batch)."""
    import torch

    from sfem_gb300.batch import BatchSolver

    sample = probs[::stride]
    times, ok = [], True
    for p in sample:
        bs = BatchSolver([p], device=dev)
        b = bs.rhs()
        x = torch.zeros_like(b)
        torch.cuda.synchronize()
        rc, _, _, sec = bs.solve(b, x)
        ok = ok and rc == 0 and bool((bs.true_residuals(b, x) <= 1.5e-10).all())
        times.append(sec)
        del bs, b, x
    t = np.asarray(times)
    # served back to back in draw order, every problem submitted at t = 0
    done = np.cumsum(t)
    return {
        "sample": f"every {stride}th of the {len(probs)} problems ({len(sample)} solves), same problems and rhs",
        "all_converged": bool(ok), "seconds_sum": float(t.sum()), "solves_per_s": len(t) / float(t.sum()),
        "solve_s_p50": float(np.percentile(t, 50)), "solve_s_p99": float(np.percentile(t, 99)),
        "queue_latency_p50_s_scaled_to_all": float(np.percentile(done, 50)) * stride,
        "queue_latency_p99_s_scaled_to_all": float(np.percentile(done, 99)) * stride,
    }


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)

    from sfem_gb300 import capi
    from sfem_gb300.operators import Laplacian, SSMeshDevice

    capi.load()
    m = workload_config(args.nx)
    sp = SSMeshDevice(m, LEVEL, device=dev)
    op = Laplacian(sp).initialize()
    N, E = m.n_nodes(), m.n_elements
    x64 = torch.randn(N, dtype=torch.float64, device=dev, generator=torch.Generator(device=dev).manual_seed(1))
    x = x64.float()
    y = torch.zeros(N, dtype=torch.float32, device=dev)
    flush = L2Flush(dev)
    stream = torch.cuda.current_stream(dev)

    for _ in range(max(3, args.warmup)):
        y.zero_()
        op.apply(x, y)
    torch.cuda.synchronize()
    # device-timed region: events around each apply (the y.zero_ is the
    # accumulate-interface's caller-side reset and is excluded), L2 flushed after the reset
    # and before each step, so x, y, connectivity and metric all come from HBM
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        wall0 = time.perf_counter()
        for k in range(args.steps):
            y.zero_()
            flush(k)  # after the reset, so y too comes from HBM
            starts[k].record(stream)
            op.apply(x, y)
            ends[k].record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    times = [s_.elapsed_time(e_) for s_, e_ in zip(starts, ends)]
    value, t_kernel = replica_aggregate(float(np.mean(times)) / 1e3, N, world, dev)
    value /= 1e9

    # end-to-end through the C ABI with host buffers: every step copies its x from pinned
    # host memory, resets y, applies (the operator's FP32 apply from its packed tiles,
    # sfem_gb300_sshex8_laplacian_apply_packed, on an explicit stream) and copies y back to
    # pinned host memory.  Consecutive steps overlap on three streams (host-to-
    # device, compute, device-to-host) with double-buffered device and host buffers.
    e2e_value, t_e2e = measure_e2e(op, x, N, max(20, args.steps), world, dev)

    # FP64 apply on the same mesh (oracle-parity precision)
    y64 = torch.zeros(N, dtype=torch.float64, device=dev)
    t64 = time_apply(op, x64, y64, args.steps, args.warmup, flush, stream)
    del flush

    solve = None
    if not args.no_solve:
        solve = {"poisson_sshex8_L4_48cube": measure_solves(m, dev),
                 "elasticity_sshex8_L4_64x16x16": measure_elasticity_solves(dev)}
        if not args.no_learned:
            solve["learned_smoother_32cube"] = measure_learned(dev)
        if not args.no_batch:
            solve["batched_serving"] = measure_batch(dev, args.batch_problems)

    peak, peak_kind = measured_peak_hbm()
    # compulsory bytes of y += A x through the accumulate interface: x read, y read and
    # written (the caller's reset is a separate pass), connectivity and FFF read once
    alg_bytes = 3 * 4 * N + (4 * (LEVEL + 1) ** 3 + 24) * E
    alg_bytes64 = 3 * 8 * N + (4 * (LEVEL + 1) ** 3 + 24) * E
    achieved = alg_bytes / t_kernel / 1e9
    fp64_flops = 2 * stencil_fma_per_element(LEVEL) * E  # node-centric form, 2 flop per tap
    line = {
        "metric": METRIC,
        "value": value, "unit": "GDoF/s", "n_gpus": world, "steps": args.steps, "warmup": max(3, args.warmup),
        "ms_per_step": t_kernel * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_dict(m, world),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": TRAFFIC_BYTES_PER_LAUNCH, "peak_kind": peak_kind, "algorithmic_bytes": alg_bytes},
        "e2e": {"value": e2e_value, "unit": "GDoF/s", "h2d_bytes_per_step": 4 * N, "d2h_bytes_per_step": 4 * N},
        "fp64_apply": {"gdofs": N / t64 / 1e9, "ms": t64 * 1e3, "achieved_gbs": alg_bytes64 / t64 / 1e9,
                       "fp64_tflops": fp64_flops / t64 / 1e12,
                       "fp64_frac_of_nominal": fp64_flops / t64 / 1e12 / NOMINAL_FP64_TFLOPS,
                       "bound": "fp64 pipe (FMA)"},
        "solve": solve,
        "gpu_launches": args.steps,
        "clocks": clk.summary(),
        "wall_s_timed": wall,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline(m)
            line["fp64_apply"]["cpu_port_gdofs"] = N / cpu_apply_time(m, "f64") / 1e9
        except Exception as exc:
            line["cpu_baseline"] = {"value": None, "error": str(exc)}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def profile_kernels():
    """Two launches of each main kernel on the bench workloads (48^3 L=4 Laplacian FP32 /
    FP64 apply, level 2 <-> 4 transfers, the fused learned correction on the 48^3
    patches, 64x16x16 L=4 elasticity FP32 / FP64): a target for per-kernel ncu
    captures."""
    import ctypes

    import torch

    from sfem_gb300 import capi
    from sfem_gb300 import solvers as S
    from sfem_gb300.learned import PatchNet
    from sfem_gb300.mesh import SSMesh
    from sfem_gb300.operators import Laplacian

    dev = torch.device("cuda:0")
    lib = capi.load()
    m = workload_config(NX)
    H = S.Hierarchy(m, dirichlet_faces=("x0",), device=dev)
    sp = H.spaces[0]
    op = Laplacian(sp).set_fff(H.fff)
    N = m.n_nodes()
    for dt in (torch.float32, torch.float64):
        x = torch.randn(N, dtype=dt, device=dev)
        y = torch.zeros_like(x)
        for _ in range(2):
            y.zero_()
            op.apply(x, y)
    ctx = S.context()
    P = S.prolongation_op(ctx, H.spaces[1], H.spaces[0], 1, H.dirichlet[0], torch.float32)
    R = S.restriction_op(ctx, H.spaces[0], H.spaces[1], 1, H.dirichlet[1], torch.float32)
    xc = torch.randn(H.spaces[1].n_nodes, dtype=torch.float32, device=dev)
    xf = torch.randn(N, dtype=torch.float32, device=dev)
    for _ in range(2):
        S.apply(P, xc, xf)
        S.apply(R, xf, xc)
    net = PatchNet(dev, seed=0)
    frag = torch.empty(lib.sfem_gb300_learned_fragments_size(), dtype=torch.uint8, device=dev)
    capi.check(lib.sfem_gb300_learned_fragments(capi.vp(net.wbf[0]), capi.vp(net.wbf[1]), capi.vp(net.wbf[2]),
                                                capi.vp(frag), None), "fragments")
    r = torch.randn(N, dtype=torch.float32, device=dev)
    inv = torch.ones_like(r)
    d = torch.zeros_like(r)
    for _ in range(2):
        capi.check(lib.sfem_gb300_learned_correction(capi.FLOAT32, capi.i64(m.n_elements), sp.lidx_ptrs.ptr,
                                                     capi.vp(r), capi.vp(inv), capi.vp(frag), capi.vp(sp.count),
                                                     ctypes.c_double(1.0), capi.vp(d), None), "learned")
    del H, op
    me = SSMesh(64, 16, 16, LEVEL, box=((0, 4), (0, 1), (0, 1)))
    He = S.Hierarchy(me, dirichlet_faces=("x0",), device=dev, vec=3)
    for dt in (torch.float32, torch.float64):
        ope = S.elasticity_op(ctx, He.spaces[0], He.adj, He.det, 1.0, 10.0, He.dirichlet[0], dt)
        u = torch.randn(3 * me.n_nodes(), dtype=dt, device=dev)
        v = torch.zeros_like(u)
        for _ in range(2):
            v.zero_()
            S.apply(ope, u, v)
    torch.cuda.synchronize()
    print("profile kernels: done")


def profile_apply():
    """Two launches each of the 48^3 L=4 Laplacian applies from packed tiles: the FP32
    stencil kernel (the step), the FP32 element-matrix kernel and the FP64 stencil
    kernel; then two each of the FP32 and FP64 stencil applies at L=3 from SoA rows on
    a 64^3 macro mesh (7,189,057 nodes).  A small ncu target (about 150 MB of inputs per
    apply, above the L2)."""
    import torch

    from sfem_gb300 import capi
    from sfem_gb300.mesh import SSMesh
    from sfem_gb300.operators import Laplacian, SSMeshDevice

    dev = torch.device("cuda:0")
    lib = capi.load()
    m = workload_config(NX)
    op = Laplacian(SSMeshDevice(m, LEVEL, device=dev)).initialize()
    N = m.n_nodes()
    for dt, variant in ((torch.float32, -1), (torch.float32, 3), (torch.float64, -1)):
        x = torch.randn(N, dtype=dt, device=dev)
        y = torch.zeros_like(x)
        prev = lib.sfem_gb300_set_laplacian_kernel(variant)
        for _ in range(2):
            y.zero_()
            op.apply(x, y)
        lib.sfem_gb300_set_laplacian_kernel(prev)
    del op
    m3 = SSMesh(64, 64, 64, 3, perturb=PERTURB, seed=SEED)
    op3 = Laplacian(SSMeshDevice(m3, 3, device=dev), packed=False).initialize()
    for dt in (torch.float32, torch.float64):
        x = torch.randn(m3.n_nodes(3), dtype=dt, device=dev)
        y = torch.zeros_like(x)
        for _ in range(2):
            y.zero_()
            op3.apply(x, y)
    torch.cuda.synchronize()
    print("profile apply: done")


def profile_zoo():
    """Two launches of each remaining kernel family on inputs larger than the 126 MB L2:
    the BLAS / CG / Chebyshev / precision-bridge vector kernels on 40M-entry vectors,
    the Dirichlet copy, the symmetric CRS and 3x3 BSR SpMV and the matrix-free hex8
    Laplacian on a 96^3 hex8 mesh (912,673 nodes), the L=2 thread-per-element and
    L=3 staged float sshex8 kernels on 96^3 / 64^3 macro meshes, the elasticity applies
    of the L=2 and hex8 levels of the 64x16x16 cantilever, and the dense coarse-level
    mat-vec (1536 unknowns)."""
    import ctypes

    import torch

    from sfem_gb300 import capi
    from sfem_gb300 import solvers as S
    from sfem_gb300.mesh import SSMesh, upper_crs_graph
    from sfem_gb300.operators import Laplacian, SSMeshDevice

    dev = torch.device("cuda:0")
    lib = capi.load()
    D = ctypes.c_double
    ws = torch.zeros(lib.sfem_gb300_reduce_workspace_size(), dtype=torch.uint8, device=dev)
    sc = torch.ones(8, dtype=torch.float64, device=dev)
    n = 40_000_000
    for dt, rt in ((torch.float64, capi.FLOAT64), (torch.float32, capi.FLOAT32)):
        x, y, z, w = (torch.rand(n, dtype=dt, device=dev) + 0.5 for _ in range(4))
        for _ in range(2):
            capi.check(lib.sfem_gb300_dot(rt, capi.i64(n), capi.vp(x), capi.vp(y), capi.vp(ws), capi.vp(sc), None), "dot")
            capi.check(lib.sfem_gb300_axpby(rt, capi.i64(n), D(0.5), capi.vp(x), D(0.5), capi.vp(y), None), "axpby")
            capi.check(lib.sfem_gb300_zaxpby(rt, capi.i64(n), D(0.5), capi.vp(x), D(0.5), capi.vp(y), capi.vp(z), None),
                       "zaxpby")
            capi.check(lib.sfem_gb300_xypaz(rt, capi.i64(n), capi.vp(x), capi.vp(y), D(0.5), capi.vp(z), None), "xypaz")
            capi.check(lib.sfem_gb300_cg_update_x_r(rt, capi.i64(n), capi.vp(sc), capi.c_void(sc.data_ptr() + 8),
                                                     capi.vp(x), capi.vp(y), capi.vp(z), capi.vp(w), capi.vp(ws),
                                                     capi.c_void(sc.data_ptr() + 16), None), "cg_update_x_r")
            capi.check(lib.sfem_gb300_cg_update_p(rt, capi.i64(n), capi.vp(sc), capi.c_void(sc.data_ptr() + 8), None,
                                                   capi.vp(x), capi.vp(y), None), "cg_update_p")
            capi.check(lib.sfem_gb300_chebyshev_update(rt, capi.i64(n), D(0.1), D(0.5), capi.vp(w), capi.vp(x),
                                                        capi.vp(y), capi.vp(z), capi.vp(w), None), "chebyshev_update")
        del x, y, z, w
    x64 = torch.rand(n, dtype=torch.float64, device=dev)
    y32 = torch.rand(n, dtype=torch.float32, device=dev)
    nodes = torch.randperm(n // 4, device=dev)[: n // 40].to(torch.int32).sort().values
    for _ in range(2):
        capi.check(lib.sfem_gb300_scaled_to_f32(capi.i64(n), capi.vp(sc), capi.vp(x64), capi.vp(y32), None), "to_f32")
        capi.check(lib.sfem_gb300_scaled_axpy_f32_to_f64(capi.i64(n), capi.vp(sc), capi.vp(y32), capi.vp(x64), None),
                   "axpy_f32_to_f64")
        capi.check(lib.sfem_gb300_constraint_nodes_copy(capi.FLOAT64, capi.i64(nodes.numel()), capi.vp(nodes), 4, 0,
                                                         capi.vp(x64), capi.c_void(x64.data_ptr()), None),
                   "constraint copy")
    del x64, y32
    # hex8 Laplacian on 96^3 elements: matrix-free apply, CRS assembly, symmetric CRS and BSR SpMV
    m = SSMesh(96, 96, 96, 1, perturb=0.1)
    sp = SSMeshDevice(m, 1, device=dev)
    lap = Laplacian(sp).initialize()
    N = m.n_nodes(1)
    rowptr, colidx = upper_crs_graph(m.hex8_elements(), N)
    rp = torch.from_numpy(rowptr).to(dev)
    ci = torch.from_numpy(colidx).to(dev)
    nnz = int(colidx.size)
    for dt, rt in ((torch.float64, capi.FLOAT64), (torch.float32, capi.FLOAT32)):
        xv = torch.rand(N, dtype=dt, device=dev)
        yv = torch.zeros_like(xv)
        diag = torch.zeros(N, dtype=dt, device=dev)
        off = torch.zeros(nnz, dtype=dt, device=dev)
        capi.check(lib.sfem_gb300_hex8_laplacian_crs_sym(capi.i64(m.n_elements), sp.elements_ptrs.ptr, capi.i64(m.n_elements),
                                                          capi.vp(lap.fff), capi.vp(rp), capi.vp(ci), rt, capi.vp(diag),
                                                          capi.vp(off), None), "crs assembly")
        for _ in range(2):
            lap.apply(xv, yv)
            capi.check(lib.sfem_gb300_crs_sym_spmv(rt, capi.i64(N), capi.vp(rp), capi.vp(ci), capi.vp(diag), capi.vp(off),
                                                    D(0.0), capi.vp(xv), capi.vp(yv), None), "crs spmv")
        del xv, yv, diag, off
    bx = torch.rand(3 * N, dtype=torch.float64, device=dev)
    by = torch.zeros_like(bx)
    bd = torch.rand(6 * N, dtype=torch.float64, device=dev)
    bo = torch.rand(9 * nnz, dtype=torch.float64, device=dev) * 1e-3
    for _ in range(2):
        capi.check(lib.sfem_gb300_bsr_sym_spmv(capi.FLOAT64, 3, capi.i64(N), capi.vp(rp), capi.vp(ci), capi.vp(bd),
                                                capi.vp(bo), 0, D(0.0), capi.vp(bx), capi.vp(by), None), "bsr spmv")
    del bx, by, bd, bo, lap, sp
    # float sshex8 kernels of the coarser levels: L=2 (thread per element) and L=3 (staged tile)
    for L, nx in ((2, 96), (3, 64)):
        ms = SSMesh(nx, nx, nx, L, perturb=0.1)
        sps = SSMeshDevice(ms, L, device=dev)
        ops = Laplacian(sps).initialize()
        xs = torch.rand(ms.n_nodes(L), dtype=torch.float32, device=dev)
        ys = torch.zeros_like(xs)
        for _ in range(2):
            ops.apply(xs, ys)
        del ops, sps, xs, ys
    # elasticity on the levels of the 64x16x16 cantilever hierarchy below L=4: L=2 and the hex8
    # macro mesh (SIMT kernels, FP32 and FP64; compute bound)
    for L in (2, 1):
        me = SSMesh(64, 16, 16, L, box=((0, 4), (0, 1), (0, 1)))
        He = S.Hierarchy(me, dirichlet_faces=("x0",), device=dev, vec=3, coarsen_macro=False)
        ctx_e = S.context()
        for dt in (torch.float32, torch.float64):
            ope = S.elasticity_op(ctx_e, He.spaces[0], He.adj, He.det, 1.0, 10.0, He.dirichlet[0], dt)
            u = torch.rand(3 * me.n_nodes(L), dtype=dt, device=dev)
            v = torch.zeros_like(u)
            for _ in range(2):
                S.apply(ope, u, v)
        del He
    # dense coarse-level solve (1536 unknowns): a hex8 Poisson level of 15 x 15 x 5 elements
    mc = SSMesh(15, 15, 5, 1)
    Hc = S.Hierarchy(mc, dirichlet_faces=("x0",), device=dev, coarsen_macro=False)
    ctx = S.context()
    opc = S.laplacian_op(ctx, Hc.spaces[0], Hc.fff, Hc.dirichlet[0], torch.float32)
    dsol = S.dense_solver(ctx, opc)
    bc = torch.rand(Hc.spaces[0].n_nodes, dtype=torch.float32, device=dev)
    xc = torch.zeros_like(bc)
    for _ in range(2):
        S.apply(dsol, bc, xc)
    torch.cuda.synchronize()
    print("profile zoo: done")


def profile_solves():
    """One FP64 flexible-CG solve preconditioned by the FP32 multigrid with the learned
    correction (32^3 L=4, k = exp(g), untrained network, 12 iterations) and one
    mixed-precision elasticity solve (64x16x16 L=4, to 1e-9); V-cycles graph-replayed."""
    import torch

    from sfem_gb300 import learned
    from sfem_gb300 import solvers as S
    from sfem_gb300.coefficients import lognormal_coefficient
    from sfem_gb300.mesh import SSMesh

    dev = torch.device("cuda:0")
    nx = 32
    mesh = SSMesh(nx, nx, nx, LEVEL)
    H = learned.hierarchy_with_coefficient(mesh, lognormal_coefficient(nx, nx, nx, ell=8.0, sigma=1.0, seed=5000), dev)
    net = learned.PatchNet(dev, seed=0)
    g = torch.Generator(device=dev).manual_seed(0)
    b = torch.randn(H.spaces[0].n_nodes, dtype=torch.float64, device=dev, generator=g)
    b[H.dirichlet[0].long()] = 0
    ctx = S.context()
    mg, _ = learned.learned_mg(ctx, H, net, torch.float32, chain="before", coarse="dense", graph=True, fallback_sweeps=1)
    op64 = S.laplacian_op(ctx, H.spaces[0], H.spaces[0].fff, H.dirichlet[0], torch.float64)
    solver = S.cg(ctx, op64, S.mixed_precond(ctx, mg), rtol=1e-10, max_it=12, residual_norm=True, flexible=True)
    for _ in range(2):
        x = torch.zeros_like(b)
        S.solve(solver, b, x)
    torch.cuda.synchronize()
    del mg, solver, H
    me = SSMesh(64, 16, 16, LEVEL, box=((0, 4), (0, 1), (0, 1)), perturb=0.0, seed=SEED)
    He = S.Hierarchy(me, dirichlet_faces=("x0",), device=dev, vec=3, coarsen_macro=True)
    mge, _ = S.build_elasticity_mg(ctx, He, torch.float32, coarse="dense", graph=True)
    ope = S.elasticity_op(ctx, He.spaces[0], He.adj, He.det, 1.0, 10.0, He.dirichlet[0], torch.float64)
    fe = torch.from_numpy(lumped_body_force(me, He.det.cpu().numpy())).to(dev)
    for c in range(3):
        fe[3 * He.dirichlet[0].long() + c] = 0
    solver = S.cg(ctx, ope, S.mixed_precond(ctx, mge), rtol=1e-9, max_it=60, residual_norm=True, flexible=True)
    for _ in range(2):
        u = torch.zeros_like(fe)
        S.solve(solver, fe, u)
    torch.cuda.synchronize()
    print("profile solves: done")


def main():
    args = parse()
    if args.profile_kernels:
        profile_kernels()
        return
    if args.profile_apply:
        profile_apply()
        return
    if args.profile_solves:
        profile_solves()
        return
    if args.profile_zoo:
        profile_zoo()
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
