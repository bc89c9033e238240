#!/usr/bin/env python3
"""Headline benchmark of the fhhos4 solve phase on GB300.

Workload: the reference's "plain method at scale" problem: 3D Poisson on the unit cube,
64^3 cubes x 6 tetrahedra, HHO k=1 (3 DOFs per face, 9,363,456 unknowns), identity tensor,
f = 3 pi^2 prod sin(pi x_i), homogeneous Dirichlet; FCG(1) preconditioned by one geometric
multigrid V(1,1) cycle with block Gauss-Seidel (bgs/rbgs), coarsest direct solve, stop at
1e-8 relative residual. The hierarchy is produced on the host by fhhos4_gb300.hho (the
reference's discretisation, validated against it) and uploaded once.

One step = one complete solve to 1e-8 with b resident in HBM. `value` = seconds per solve of
the learned step + FP32 V-cycle inside the FP64-class FCG; the plain method (the reference's
V(1,1), same iteration count) is reported beside it in FP32-pair (FP64-class) and native FP64
arithmetic. `e2e` = the same solve through the C ABI with host buffers (H2D of b, D2H of x inside
the timed region). Beside the headline, in the same line: the 48^3 k = 2 checkerboard (contrast
1e6) workload, the 32^3 rotated-anisotropic workload (plain, FP32 and learned, with rediscretised
and Galerkin coarse operators), the 512-problem batched workload (2D, uneven sizes, one graph
launch), the GPU condensation and post-processing of the headline system; `--no-extra` and
`--extra` select.

--impl reference times the reference's CPU algorithm (the oracle restatement, natural block-GS
order, OpenMP row-parallel products) on the host cores, one step = one FCG iteration, scaled
to the reference's iteration count.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "s to 1e-8 FP64 rel residual: learned+FP32 MG-FCG vs plain FP64; SpMV GB/s"
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--dim", type=int, default=3)
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--k", type=int, default=1)
    ap.add_argument("--coefficient", default="identity", choices=["identity", "checkerboard", "anisotropic",
                                                                  "lognormal_patches"])
    ap.add_argument("--contrast", type=float, default=1e6)
    ap.add_argument("--source", default="sine", choices=["sine", "one"])
    ap.add_argument("--max-coarse-rows", type=int, default=1000)
    ap.add_argument("--galerkin", action="store_true", help="Galerkin coarse operators (the reference's -g 1)")
    ap.add_argument("--replace-residual", action="store_true",
                    help="residual replacement in every precision (FP64 true residual, compensated when it misses tol)")
    ap.add_argument("--fast-smoothers", default="bgs,rbgs", help="pre,post smoothers of the fast (FP32) method")
    ap.add_argument("--fast-nu", default="3,3", help="pre,post smoothing steps of the fast (FP32) method")
    ap.add_argument("--fast-coarse-nu", default="4,4",
                    help="pre,post smoothing steps of the fast method on levels >= 1 (-1,-1: as --fast-nu)")
    ap.add_argument("--weights", default="", help="learned-step network (default: the committed one)")
    ap.add_argument("--no-learned", action="store_true", help="report the FP32 method as the headline")
    ap.add_argument("--batch", type=int, default=0,
                    help="also run the batched workload: this many 2D problems in one graph launch")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="only the headline (tet 64^3, k = 1): skip the other workloads and the 512-problem batch")
    ap.add_argument("--batch-precisions", default="fp32",
                    help="V-cycle precisions of the batched workload (fp32, df; each sets up all problems again)")
    ap.add_argument("--extra", default="",
                    help="only these extra workloads (comma-separated keys, e.g. tet32_k1_anisotropic); no batch unless --batch")
    ap.add_argument("--cpu-sample-iterations", type=int, default=2)
    return ap.parse_args()


# --------------------------------------------------------------------------- distributed
class Dist:
    """One process per GPU (torchrun); replicas: every rank solves its own copy."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local_rank)
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        dev = "cuda" if torch.cuda.is_available() else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during a timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        # "under load": samples within 40% of the highest power seen
        pmax = max(power)
        loaded = [s for s, p in zip(sm, power) if p >= 0.6 * pmax] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": pmax}


def log(msg: str):
    """Progress of the bench on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def measured_hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def committed_traffic():
    """dram bytes per launch of the profiled kernels (profiles/traffic.json), if committed."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# --------------------------------------------------------------------------- workload
def workload_config(args, unknowns=None, levels=None):
    """The workload, identical in both arms (the problem and the stopping test; the solver method
    of each arm is reported beside it, not in it)."""
    coef = "identity tensor" if args.coefficient == "identity" else (
        f"{args.coefficient} coefficient (contrast {args.contrast:g})")
    name = (f"{'3D tet' if args.dim == 3 else '2D tri'} {args.n}^{args.dim} HHO k={args.k} diffusion, {coef}, "
            f"f={'sine' if args.source == 'sine' else '1'}, solved to 1e-8 FP64 relative residual")
    cfg = {"workload": name, "dim": args.dim, "n": args.n, "k": args.k, "mesh": "stetra" if args.dim == 3 else "stri",
           "coefficient": args.coefficient, "source": args.source, "tolerance": 1e-8,
           "coarse_operators": "Galerkin P^T A P (-g 1)" if args.galerkin else "rediscretised (the reference default)",
           "max_coarse_rows": args.max_coarse_rows,
           "l2": "inputs larger than L2 (fine operator alone is > 1 GB)" if args.n >= 48 else
                 "operators of every level together larger than L2"}
    if unknowns is not None:
        cfg["unknowns"] = int(unknowns)
    if levels is not None:
        cfg["levels"] = int(levels)
    return cfg


def checker_blocks(args):
    """Blocks per direction of the coefficient field: 4 x 4 x 4 for the checkerboard, one block per
    4^3 cubes for the rotated anisotropic tensor, 8 x 8 patches for the log-uniform field."""
    if args.coefficient == "anisotropic":
        return max(1, args.n // 4)
    if args.coefficient == "lognormal_patches":
        return 8
    return 4


def generate(args, keep=False):
    from fhhos4_gb300 import hho
    t0 = time.perf_counter()
    H = hho.Hierarchy(args.dim, args.n, args.k, coefficient=args.coefficient, contrast=args.contrast,
                      source=args.source, max_coarse_rows=args.max_coarse_rows, checker_blocks=checker_blocks(args),
                      seed=getattr(args, "seed", 20261203))
    As = [H.A(l) for l in range(H.levels)]
    Ps = [H.P(l) for l in range(H.levels - 1)]
    b = H.b()
    bs = H.block_size
    dt = time.perf_counter() - t0
    if not keep:
        H.close()
        H = None
    return As, Ps, b, bs, dt, H


def reference_iterations(args):
    """Iterations of the reference (natural order) and of the reference in colour order, from the
    committed reference histories when present."""
    if args.coefficient != "identity" or args.source != "sine" or args.dim != 3:
        return None, None
    try:
        z = np.load(os.path.join(ROOT, "tests", "golden", f"tet3d_n{args.n}_k{args.k}.npz"))
        return len(z["hist_natural"]) - 1, len(z["hist_colour"]) - 1
    except (OSError, KeyError):
        return None, None


def cpu_sample(As, Ps, b, bs, iters: int, threads: int):
    """Seconds per FCG iteration of the oracle restatement (setup excluded) on `threads` cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.set_threads(threads)
    x, hist, it, rc = O.fcgmg_solve(As, Ps, b, bs, maxit=iters, tol=0.0)
    setup_s, iter_s = O.last_timing()
    return iter_s / max(it, 1), setup_s, it


def bytes_spmv(nnzb, nb_rows, n_in, n_out, bs, p, residual=False, add=False):
    """Algorithmic bytes of one BSR product: values + column indices + row pointers + x read once
    + y written (+ b or the added vector read)."""
    b = nnzb * bs * bs * p + nnzb * 4 + (nb_rows + 1) * 4 + n_in * p + n_out * p
    if residual or add:
        b += n_out * p
    return b


def measure_methods(ctx, dist, dev, b_dev, x_dev, maxit, methods, warmup, steps, params=None, wmeta=None, bs=3):
    """Solve b (resident on the device) with every method on one context: `warmup` untimed solves, then
    `steps` timed ones (CUDA events on the library's stream, max over ranks). methods: name ->
    (precision, pre, post, npre, npost, (coarse npre, coarse npost), learned), learned False, True (the
    fallback rule) or "always"."""
    import torch
    results, launches, clocks, solutions = {}, {}, {}, {}
    for name, (prec, pre, post, npre, npost, coarse, use_learned) in methods.items():
        ctx.set_cycle(pre, post, npre, npost, 1)
        ctx.set_coarse_smoothing(*coarse)
        ctx.set_vcycle_precision(prec)
        if use_learned:
            ctx.set_learned(params, use_learned if isinstance(use_learned, str) else "fallback")
        elif bs <= 4 and params is not None:
            ctx.set_learned(None, "off")

        def solve_device():
            rc, hist, info = ctx.solve_device(b_dev.data_ptr(), x_dev.data_ptr(), maxit)
            if rc != 0:
                ctx._check(rc)
            return hist, info

        for _ in range(warmup):
            solve_device()
        dist.barrier()
        torch.cuda.synchronize()
        sampler = ClockSampler(dev)
        sampler.start()
        k0 = ctx.kernel_launches()
        times, iters = [], []
        for _ in range(steps):
            hist, info = solve_device()
            times.append(info.solve_ms / 1e3)
            iters.append(info.iterations)
        torch.cuda.synchronize()
        launches[name] = ctx.kernel_launches() - k0
        clocks[name] = sampler.stop()
        dist.barrier()
        t_step = dist.max(float(np.mean(times)))
        solutions[name] = x_dev.cpu().numpy()
        results[name] = dict(s=t_step, iterations=iters[-1], true_rel_residual=info.true_relative_residual,
                             final=float(hist[-1]),
                             cycle=f"V({npre},{npost}) {pre}/{post}" + (
                                 f", V({coarse[0]},{coarse[1]}) on levels >= 1" if min(coarse) >= 0 else ""),
                             vcycle_precision=prec)
        if use_learned:
            results[name]["learned_iterations"] = info.learned_iterations
            results[name]["fallback_reference_rate"] = ctx.learned_reference_rate()
            results[name]["network"] = wmeta
    return results, launches, clocks, solutions


def gpu_post_processing(H, x, dev):
    """Cell unknowns and the L2 error of the k+1 reconstruction of the headline solution on the GPU
    (fhg_post_run), beside the host's evaluation of the same x."""
    import torch
    from fhhos4_gb300 import _native as N
    t = H.post_tables()
    post = N.Post(t, dev)
    try:
        xd = torch.from_numpy(x).to(f"cuda:{dev}")
        cells = torch.empty(t["n_elements"] * t["n_cell"], dtype=torch.float64, device=f"cuda:{dev}")
        post.run(xd.data_ptr(), cells.data_ptr(), "sine")
        err, ms = post.run(xd.data_ptr(), cells.data_ptr(), "sine")
    finally:
        post.close()
    t0 = time.perf_counter()
    host = H.l2_error(x)
    host_s = time.perf_counter() - t0
    return {"what": "cell unknowns + k+1 reconstruction + relative L2 error vs the exact solution",
            "l2_error_gpu": err, "l2_error_host": host, "gpu_ms": round(ms, 3), "host_s": round(host_s, 3),
            "elements": int(t["n_elements"]), "element_classes": int(t["n_classes"]),
            "quadrature_points": int(t["n_points"])}


def gpu_condensation(H, A0, b0, dev):
    """The finest system condensed and assembled on the GPU (fhg_cond_run) from the element tables,
    compared with the host assembly the solve uses."""
    from fhhos4_gb300 import _native as N
    t = H.condense_tables()
    cond = N.Condense(t, dev)
    try:
        cond.run()
        nnz, ms = cond.run()
        A, b = cond.result(nnz)
    finally:
        cond.close()
    same = bool(np.array_equal(A.indptr, A0.indptr) and np.array_equal(A.indices, A0.indices))
    # the coarse levels' rediscretised operators the same way
    coarse_ms, coarse_diff, coarse_same = 0.0, 0.0, True
    for l in range(1, H.levels):
        Al = H.A(l).tocsr()
        c = N.Condense(H.level_tables(l), dev)
        try:
            nnz_l, ms_l = c.run()
            Ag, _ = c.result(nnz_l)
        finally:
            c.close()
        coarse_ms += ms_l
        ok = bool(np.array_equal(Ag.indptr, Al.indptr) and np.array_equal(Ag.indices, Al.indices))
        coarse_same &= ok
        if ok:
            coarse_diff = max(coarse_diff, float(np.abs(Ag.data - Al.data).max() / np.abs(Al.data).max()))
    return {"what": "static condensation (per-class Schur complements) + assembly of A_0 and b on the GPU; "
                    "the coarse levels' rediscretised operators the same way",
            "gpu_ms": round(ms, 3), "same_structure": same,
            "max_rel_diff_A": float(np.abs(A.data - A0.data).max() / np.abs(A0.data).max()) if same else None,
            "max_rel_diff_b": float(np.abs(b - b0).max() / np.abs(b0).max()),
            "coarse_levels": H.levels - 1, "coarse_gpu_ms": round(coarse_ms, 3), "coarse_same_structure": coarse_same,
            "coarse_max_rel_diff": coarse_diff if coarse_same else None,
            "element_classes": int(t["n_classes"]), "elements": int(t["n_elements"])}


def run_ours(args, dist: Dist):
    import torch
    from fhhos4_gb300 import _native as N

    dev = dist.local_rank
    torch.cuda.set_device(dev)
    As, Ps, b, bs, gen_s, H = generate(args, keep=True)
    n0 = As[0].shape[0]
    fast_pre, fast_post = args.fast_smoothers.split(",")
    fast_npre, fast_npost = (int(v) for v in args.fast_nu.split(","))
    fast_cpre, fast_cpost = (int(v) for v in args.fast_coarse_nu.split(","))
    ctx = N.Context(dev)
    t0 = time.perf_counter()
    for l, A in enumerate(As):
        ctx.set_level(l, bs, A)
    for l, P in enumerate(Ps):
        ctx.set_prolongation(l, P)
    ctx.set_face_tensors(H.face_tensors(0))
    o = N.default_options()
    o.vcycle_precision = N.PRECISION["fp32"]   # keeps FP64 and FP32 copies
    o.extra_precisions = 1 << N.PRECISION["df"]   # and the FP32-pair copies (FP64-class V-cycle)
    o.galerkin = 1 if args.galerkin else 0
    o.replace_residual = 1 if args.replace_residual else 0
    o.autotune = 1
    o.max_iterations = 200
    ctx.setup(len(As), o)
    setup_s = time.perf_counter() - t0
    info0 = ctx.level_info(0)

    b_dev = torch.from_numpy(b).to(f"cuda:{dev}")
    x_dev = torch.empty_like(b_dev)
    torch.cuda.synchronize()

    # Methods on the same hierarchy and context:
    #   plain        the reference's method, V(1,1) bgs/rbgs, in FP64-class arithmetic: the V-cycle and
    #                the outer FCG on FP32 pairs (FHG_PREC_DF, ~2^-47 per term on the FP32 pipe), x and
    #                the Krylov scalars FP64; the reference's iteration count and history (the
    #                metric's "plain FP64");
    #   plain_native the same method in native FP64 arithmetic (bound by GB300's FP64 pipe);
    #   fp64_fast    the FP64-class V-cycle with the fast method's cycle (isolates the precision gain);
    #   fast         FP32 V-cycle inside FP64 FCG with the fast cycle;
    #   learned      the same with the learned correction in the V-cycle (fallback rule on): the
    #                headline `value` (the metric's "learned+FP32 MG-FCG").
    from fhhos4_gb300 import learned as LN
    params, wmeta = LN.load_params(args.weights or LN.DEFAULT_WEIGHTS)
    # the learned step exists for face blocks of 2..4 unknowns (k = 1 in 3D)
    have_learned = bs <= 4 and not args.no_learned
    fast_coarse = (fast_cpre, fast_cpost)
    methods = {"plain": ("df", "bgs", "rbgs", 1, 1, (-1, -1), False),
               "plain_native": ("fp64", "bgs", "rbgs", 1, 1, (-1, -1), False),
               "fp64_fast": ("df", fast_pre, fast_post, fast_npre, fast_npost, fast_coarse, False),
               "fast": ("fp32", fast_pre, fast_post, fast_npre, fast_npost, fast_coarse, False)}
    if have_learned:
        methods["learned"] = ("fp32", fast_pre, fast_post, fast_npre, fast_npost, fast_coarse, True)
    results, launches, clocks, solutions = measure_methods(ctx, dist, dev, b_dev, x_dev, o.max_iterations, methods,
                                                           args.warmup, args.steps, params, wmeta, bs)
    x64 = solutions["plain"]
    for name in methods:
        results[name]["rel_diff_vs_plain_fp64"] = float(np.linalg.norm(solutions[name] - x64) / np.linalg.norm(x64))
        if args.source == "sine" and H is not None:
            results[name]["l2_error_vs_exact"] = H.l2_error(solutions[name])
    post_info = cond_info = None
    if args.source == "sine" and H is not None:
        post_info = gpu_post_processing(H, solutions["learned" if have_learned else "fast"], dev)
    if H is not None:
        cond_info = gpu_condensation(H, As[0], b, dev)
    if H is not None:
        H.close()

    head = "learned" if have_learned else "fast"
    # End to end through the public C ABI with pinned host buffers (H2D b, solve, D2H x), headline method.
    ctx.set_cycle(fast_pre, fast_post, fast_npre, fast_npost, 1)
    ctx.set_coarse_smoothing(fast_cpre, fast_cpost)
    ctx.set_vcycle_precision("fp32")
    if head == "learned":
        ctx.set_learned(params, "fallback")
    elif bs <= 4:
        ctx.set_learned(None, "off")
    b_host = torch.from_numpy(b).pin_memory()
    x_host = torch.empty_like(b_host).pin_memory()
    lib = N.load()
    import ctypes as C

    def solve_host():
        info = N.SolveInfo()
        rc = lib.fhg_solve(ctx.h, C.c_void_p(b_host.data_ptr()), C.c_void_p(x_host.data_ptr()), None, C.byref(info))
        if rc != 0:
            ctx._check(rc)
        return info

    for _ in range(args.warmup):
        solve_host()
    dist.barrier()
    e2e_times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        solve_host()
        e2e_times.append(time.perf_counter() - t)
    e2e_s = dist.max(float(np.mean(e2e_times)))

    # Which part of the headline cycle runs as one cluster launch (chosen by timing at setup), and the
    # context's device memory.
    first, ctas, threads = ctx.fused_coarse_info("fp32")
    fused_info = {"first_level": first, "cluster_ctas": ctas, "cta_threads": threads,
                  "device_gb": round(ctx.device_bytes() / 1e9, 2)}

    # Per-kernel device timing on level 0 (CUDA events on the library's stream).
    p32, p64 = 4, 8
    info1 = ctx.level_info(1) if len(As) > 1 else None
    nb0, nnzb0 = info0["block_rows"], info0["blocks"]
    n1 = As[1].shape[0] if len(As) > 1 else 0
    kernels = {}

    def add_kernel(name, op, prec, bytes_):
        ms = ctx.time_op(0, op, prec, warmup=3, reps=20)
        kernels[name] = {"ms": ms, "bytes": bytes_, "gbs": bytes_ / (ms * 1e-3) / 1e9}

    # outer FCG operator: double-FP32 (values as FP32 pairs, d as an FP32 pair, r.d, d.Ad; the product
    # of both the FP32 and the FP64-class methods) and native FP64
    outer_bytes = bytes_spmv(nnzb0, nb0, n0, n0, bs, 8) + n0 * 8 * 2   # + d (own rows) and r for the dots
    add_kernel("bsr_outer_dots_fp64", N.OP_SYM_SPMV, "df", outer_bytes)
    add_kernel("bsr_outer_dots_fp64_native", N.OP_SYM_SPMV, "fp64", outer_bytes)
    # FP64 operators: "fp64" = the FP64-class pair kernels the plain method runs (8-byte values);
    # "fp64_native" = the same products in native FP64 arithmetic
    for name, prec, p in (("fp32", "fp32", p32), ("fp64", "df", p64), ("fp64_native", "fp64", p64)):
        add_kernel(f"bsr_spmv_{name}", N.OP_SPMV, prec, bytes_spmv(nnzb0, nb0, n0, n0, bs, p))
        gs_bytes = bytes_spmv(nnzb0, nb0, n0, n0, bs, p) + nb0 * bs * bs * p + n0 * p   # + D^-1 + b
        add_kernel(f"bsr_gs_sweep_{name}", N.OP_GS_FORWARD, prec, gs_bytes)
        if info1:
            pb = info0["p_blocks"]
            add_kernel(f"bsr_restrict_{name}", N.OP_RESTRICT, prec, bytes_spmv(pb, n1 // bs, n0, n1, bs, p))
            add_kernel(f"bsr_prolong_add_{name}", N.OP_PROLONG_ADD, prec,
                       bytes_spmv(pb, nb0, n1, n0, bs, p, add=True))
    # The learned step (FP32 residual, block-diagonal scaling, 48-128-128-16 MLP on the tensor
    # cores) and its MLP work: 2 (48 x 128 + 128 x 128 + 128 x 16) FLOP per face.
    if have_learned:
        for kname in ("tcgen05", "mma_sync"):
            ctx.set_learned(params, "always", kernel=kname)
            ms = ctx.time_op(0, N.OP_LEARNED_STEP, "fp32", warmup=3, reps=20)
            flops = 2.0 * (48 * 128 + 128 * 128 + 128 * 16) * nb0
            kernels[f"learned_step_{kname}"] = {"ms": ms, "bytes": 0, "gbs": 0.0,
                                                "tflops_mlp": flops / (ms * 1e-3) / 1e12}
        ctx.set_learned(params, "fallback")
    # Dominant kernel of the headline (FP32 V-cycle) solve: GS sweeps on level 0.
    ncol = info0["colours"]
    gs_min_bytes = (nnzb0 - nb0) * (bs * bs * p32 + 4) + nb0 * bs * bs * p32 + 3 * n0 * p32
    dom = "bsr_gs_sweep_fp32"
    hbm, hbm_kind = measured_hbm_peak()
    traffic = committed_traffic().get(dom)
    ach = kernels[dom]["gbs"]
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(ach / hbm, 4), "peak_kind": f"of {hbm_kind}",
                "traffic": traffic,
                "algorithmic_bytes_per_launch": kernels[dom]["bytes"] / max(ncol, 1),
                "launches_per_sweep": ncol,
                # The sweep's own minimum: off-diagonal blocks with their column indices, D^-1, b,
                # x read once and written once (the formula above also counts the diagonal blocks
                # and row pointers, which the sweep does not read).
                "min_bytes_per_launch": gs_min_bytes / max(ncol, 1),
                "frac_min_bytes": round(gs_min_bytes / (kernels[dom]["ms"] * 1e-3) / 1e9 / hbm, 4),
                "spmv_fp64_frac": round(kernels["bsr_spmv_fp64"]["gbs"] / hbm, 4),
        "spmv_fp64_native_frac": round(kernels["bsr_spmv_fp64_native"]["gbs"] / hbm, 4),
                "spmv_fp32_frac": round(kernels["bsr_spmv_fp32"]["gbs"] / hbm, 4)}

    cpu = None
    ref_nat, ref_col = reference_iterations(args)
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        per_it, cpu_setup, k = cpu_sample(As, Ps, b, bs, args.cpu_sample_iterations, threads)
        its = ref_nat or results["plain"]["iterations"]
        cpu = {"value": round(per_it * its, 3), "unit": "s", "cores": threads, "kind": "port",
               "sample": (f"{k} FCG(1)+V(1,1) iterations of this {n0}-unknown solve by the oracle restatement "
                          f"(natural block-GS order, OpenMP row-parallel products), {per_it:.3f} s/iteration "
                          f"x {its} reference iterations; setup {cpu_setup:.1f} s excluded")}

    clk = clocks[head]
    value = results[head]["s"]
    line = {
        "metric": METRIC,
        "value": round(value, 6),
        "unit": "s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(value * 1e3, 3),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 (Krylov) / f32 (V-cycle)",
        "data": (f"synthetic: the reference's own {args.n}^{args.dim} HHO system ({args.coefficient} coefficient), "
                 "generated on the host"),
        "config": workload_config(args, n0, len(As)),
        "parallelism": f"replicas x{dist.world}" if dist.world > 1 else "1 GPU",
        "method": {"name": ("learned correction + " if head == "learned" else "") + "FP32 V-cycle inside FP64 FCG(1)",
                   "krylov": "FCG(1), double-FP32 outer product, FP64 x and Krylov scalars",
                   "cycle": results[head]["cycle"], "vcycle_precision": "fp32",
                   "coarsest": "FP64 dense inverse of the coarsest operator", "colours_level0": ncol,
                   "coarse_subcycle_one_launch": fused_info},
        "plain_fp64": dict(results["plain"], reference_iterations_colour_order=ref_col,
                           reference_iterations_natural_order=ref_nat,
                           arithmetic="FP64-class: FP32 pairs (~2^-47 per term) on the FP32 pipe, FP64 x"),
        "plain_fp64_native": dict(results["plain_native"], arithmetic="native FP64"),
        "fp64_fast_cycle": results["fp64_fast"],
        "fast": results["fast"],
        "learned": results.get("learned"),
        "headline_method": head,
        "speedup_vs_plain_fp64": round(results["plain"]["s"] / value, 3),
        "speedup_vs_plain_fp64_native": round(results["plain_native"]["s"] / value, 3),
        "speedup_vs_fp64_same_cycle": round(results["fp64_fast"]["s"] / value, 3),
        "learned_vs_fast": round(results["fast"]["s"] / results["learned"]["s"], 3) if have_learned else None,
        "dofs_per_s": round(n0 * dist.world / value, 1),
        "e2e": {"value": round(e2e_s, 6), "unit": "s", "h2d_bytes_per_step": int(n0 * 8),
                "d2h_bytes_per_step": int(n0 * 8)},
        "roofline": roofline,
        "kernels": {k: ({"ms": round(v["ms"], 4), "gbs": round(v["gbs"], 1), "frac": round(v["gbs"] / hbm, 4)}
                        if "tflops_mlp" not in v else {"ms": round(v["ms"], 4), "tflops_mlp": round(v["tflops_mlp"], 1)})
                    for k, v in kernels.items()},
        "gpu_launches": int(launches[head]),
        "clocks": clk,
        "setup_s": {"hierarchy_generation": round(gen_s, 2), "gpu_setup": round(setup_s, 2)},
        "condensation": cond_info,
        "post_processing": post_info,
        "cpu_baseline": cpu,
    }
    ctx.close()
    log(f"headline (tet 64^3, k = 1) done: {value * 1e3:.2f} ms")
    if not args.no_extra:
        only = [n for n in args.extra.split(",") if n] if args.extra else list(EXTRA_CONFIGS)
        for name in only:
            t = time.perf_counter()
            line[name] = run_extra(args, dist, name)
            log(f"{name} done in {time.perf_counter() - t:.1f} s")
        if not args.extra:
            args.batch = args.batch or 512
    if args.batch > 0:
        line["batched_2d_uneven"] = run_batched(args, dist)
    if dist.rank == 0:
        print(json.dumps(line), flush=True)


def run_batched(args, dist: Dist):
    """Many 2D problems of uneven size in one graph launch against the same problems solved
    one after another (fhg_solve_device each), in the V-cycle precisions of --batch-precisions (FP32
    by default; df adds the FP64-class pair V-cycle, another full setup); the contexts of one
    precision at a time (every problem's operators and views take device memory)."""
    import torch
    from fhhos4_gb300 import batch as BT
    specs = BT.batched_specs(args.batch)
    t0 = time.perf_counter()
    gen = BT.generate_all(specs)
    dofs = sum(g[1].shape[0] for g in gen)
    out = {"problems": len(specs), "unknowns": int(dofs), "n_range": [min(s.n for s in specs), max(s.n for s in specs)],
           "k_counts": {k: sum(1 for s in specs if s.k == k) for k in (1, 2, 3)},
           "method": ("V(1,1) bgs/rbgs inside FP64 FCG(1), Galerkin coarse operators, autotuned launch shapes; "
                      "residual replacement in the device loop in both precisions (compensated true residual)"),
           "host_generation_s": round(time.perf_counter() - t0, 1)}
    log(f"batched: {len(specs)} problems generated in {out['host_generation_s']} s")
    from fhhos4_gb300 import _native as N
    for prec in [q for q in args.batch_precisions.split(",") if q]:
        t1 = time.perf_counter()
        try:
            probs, batch, build_s = BT.build(specs, device=dist.local_rank, precision=prec, autotune=True, generated=gen)
        except N.FhgError as e:   # reported, not fatal: the other precision and the rest of the line go on
            out[prec] = {"error": str(e)}
            log(f"batched {prec}: setup failed: {e}")
            torch.cuda.empty_cache()
            continue
        setup_s = time.perf_counter() - t1
        device_gb = sum(p.ctx.device_bytes() for p in probs) / 1e9
        for _ in range(2):
            rc, infos, ms = batch.solve()
        times = []
        for _ in range(max(3, args.steps // 2)):
            rc, infos, ms = batch.solve()
            times.append(ms)
        batched_ms = dist.max(float(np.median(times)))
        seq_ms = 0.0
        for p in probs:
            bd = torch.from_numpy(p.b).cuda()
            xd = torch.empty_like(bd)
            torch.cuda.synchronize()
            p.ctx.solve_device(bd.data_ptr(), xd.data_ptr(), 200)
            rc1, h, info = p.ctx.solve_device(bd.data_ptr(), xd.data_ptr(), 200)
            seq_ms += info.solve_ms
            del bd, xd
        its = [i.iterations for i in infos]
        trues = sorted(i.true_relative_residual for i in infos)
        out[prec] = {"batched_ms": round(batched_ms, 2), "sequential_ms": round(seq_ms, 2),
                     "speedup_batched_vs_sequential": round(seq_ms / batched_ms, 2),
                     "dofs_per_s": round(dofs / (batched_ms * 1e-3), 1), "iterations_min_max": [min(its), max(its)],
                     "true_rel_residual_median_worst": [trues[len(trues) // 2], trues[-1]],
                     "problems_true_below_tol": sum(1 for t in trues if t < 1e-8), "status": rc,
                     "setup_s": round(setup_s, 1), "device_gb": round(device_gb, 1),
                     "timing": f"median of {max(3, args.steps // 2)} launches after 2 untimed ones"}
        log(f"batched {prec}: setup {setup_s:.1f} s ({device_gb:.1f} GB), batched {batched_ms:.1f} ms, "
            f"sequential {seq_ms:.1f} ms")
        batch.close()
        for p in probs:
            p.close()
        del probs, batch
        torch.cuda.empty_cache()
    return out


# The other workloads, measured in the same run beside the headline (tet 64^3, k = 1). Each is a
# namespace of bench options and the methods it compares; every solve is judged by its true residual.
EXTRA_CONFIGS = {
    # 48^3 tetrahedra, k = 2, 4x4x4 checkerboard 1 / 1e6, f = 1, Galerkin coarse operators,
    # residual replacement in every precision (compensated true residual where FP64 misses 1e-8).
    "tet48_k2_checkerboard_1e6": dict(dim=3, n=48, k=2, coefficient="checkerboard", contrast=1e6, source="one", max_coarse_rows=2000,
                    galerkin=True, replace_residual=True,
                    methods={"plain_fp64": ("df", "bgs", "rbgs", 1, 1, (-1, -1), False),
                             "fp64_v22": ("df", "bgs", "rbgs", 2, 2, (-1, -1), False),
                             "fp32_v22": ("fp32", "bgs", "rbgs", 2, 2, (-1, -1), False)}),
    # 32^3 tetrahedra, k = 1, diag(1, 1, eps) rotated per 4^3-cube block, eps log-uniform in
    # [1e-3, 1], a field seed the network never saw; plain, FP32 fast cycle, and the learned step (with the
    # fallback rule, and on every iteration).
    "tet32_k1_anisotropic": dict(dim=3, n=32, k=1, coefficient="anisotropic", contrast=1.0, source="one", max_coarse_rows=1000,
                    galerkin=False, replace_residual=False, seed=987654321,
                    methods={"plain_fp64": ("df", "bgs", "rbgs", 1, 1, (-1, -1), False),
                             "fp32_fast": ("fp32", "bgs", "rbgs", 3, 3, (4, 4), False),
                             "learned_fast": ("fp32", "bgs", "rbgs", 3, 3, (4, 4), True),
                             "learned_fast_always": ("fp32", "bgs", "rbgs", 3, 3, (4, 4), "always"),
                             "fp32_v22": ("fp32", "bgs", "rbgs", 2, 2, (-1, -1), False),
                             "learned_v22": ("fp32", "bgs", "rbgs", 2, 2, (-1, -1), True)}),
    # The same field with Galerkin coarse operators (the reference's -g 1): rediscretised coarse
    # operators of the rotated anisotropic field make the V-cycle a weak preconditioner.
    "tet32_k1_anisotropic_galerkin": dict(dim=3, n=32, k=1, coefficient="anisotropic", contrast=1.0, source="one",
                             max_coarse_rows=1000, galerkin=True, replace_residual=False, seed=987654321,
                             methods={"plain_fp64": ("df", "bgs", "rbgs", 1, 1, (-1, -1), False),
                                      "fp32_fast": ("fp32", "bgs", "rbgs", 3, 3, (4, 4), False),
                                      "learned_fast": ("fp32", "bgs", "rbgs", 3, 3, (4, 4), True),
                                      "learned_fast_always": ("fp32", "bgs", "rbgs", 3, 3, (4, 4), "always")}),
}
ANISO_WEIGHTS = "learned_tet3d_k1_aniso.npz"   # trained on fields of that anisotropic distribution


def run_extra(args, dist: Dist, name: str):
    """One extra configuration: host hierarchy, set-up context (FP32, pair and FP64 copies, autotuned),
    its methods timed (1 untimed and 2 timed solves each), true residuals, iterations."""
    import copy
    import torch
    from fhhos4_gb300 import _native as N
    from fhhos4_gb300 import learned as LN
    spec = dict(EXTRA_CONFIGS[name])
    methods = spec.pop("methods")
    a = copy.copy(args)
    for k, v in spec.items():
        setattr(a, k, v)
    dev = dist.local_rank
    As, Ps, b, bs, gen_s, H = generate(a, keep=True)
    ctx = N.Context(dev)
    t0 = time.perf_counter()
    for l, A in enumerate(As):
        ctx.set_level(l, bs, A)
    for l, P in enumerate(Ps):
        ctx.set_prolongation(l, P)
    ctx.set_face_tensors(H.face_tensors(0))
    H.close()
    o = N.default_options()
    o.vcycle_precision = N.PRECISION["fp32"]
    o.extra_precisions = 1 << N.PRECISION["df"]
    o.galerkin = 1 if a.galerkin else 0
    o.replace_residual = 1 if a.replace_residual else 0
    o.autotune = 1
    o.max_iterations = 300
    ctx.setup(len(As), o)
    setup_s = time.perf_counter() - t0
    params = wmeta = None
    if any(m[-1] for m in methods.values()):
        path = os.path.join(LN.WEIGHTS_DIR, ANISO_WEIGHTS)
        params, wmeta = LN.load_params(path if os.path.exists(path) else LN.DEFAULT_WEIGHTS)
    b_dev = torch.from_numpy(b).to(f"cuda:{dev}")
    x_dev = torch.empty_like(b_dev)
    torch.cuda.synchronize()
    results, launches, _, solutions = measure_methods(ctx, dist, dev, b_dev, x_dev, o.max_iterations, methods, 1, 2,
                                                      params, wmeta, bs)
    ctx.close()
    n0 = As[0].shape[0]
    ref = solutions[next(iter(methods))]
    for m in methods:
        results[m]["rel_diff_vs_plain_fp64"] = float(np.linalg.norm(solutions[m] - ref) / np.linalg.norm(ref))
        results[m]["s"] = round(results[m]["s"], 5)
        results[m]["meets_1e-8"] = bool(results[m]["true_rel_residual"] < 1e-8)
    out = {"workload": workload_config(a, n0, len(As)), "methods": results,
           "timing": "1 untimed and 2 timed solves per method, CUDA events, b resident in HBM",
           "setup_s": {"hierarchy_generation": round(gen_s, 2), "gpu_setup": round(setup_s, 2)}}
    if "learned_fast" in results:
        out["learned_vs_fast"] = round(results["fp32_fast"]["s"] / results["learned_fast"]["s"], 3)
        out["learned_always_vs_fast"] = round(results["fp32_fast"]["s"] / results["learned_fast_always"]["s"], 3)
        if "learned_v22" in results:
            out["learned_vs_fast_v22"] = round(results["fp32_v22"]["s"] / results["learned_v22"]["s"], 3)
        out["speedup_learned_vs_plain_fp64"] = round(results["plain_fp64"]["s"] / results["learned_fast"]["s"], 3)
        if not a.galerkin:
            out["energy_ratio_one_cycle"] = aniso_energy_ratios(a, dev, params)
    return out


def aniso_energy_ratios(a, dev, params, samples: int = 4):
    """|e1|_A^2 / |e|_A^2 after one V(2,2) cycle, plain and with the learned step, for seeded errors
    left by one plain cycle on the anisotropic 32^3 field (mean over `samples`)."""
    from fhhos4_gb300 import learned as LN
    f = LN.Field(LN.FieldSpec(n=a.n, seed=a.seed), device=dev, nu=(2, 2))
    try:
        f.ctx.set_learned(params, "always")
        ss = LN.make_samples(f, samples, cycles=(1,), seed=4242)
        plain = [LN.energy_ratio(f, e, False) for _, _, e in ss]
        learned = [LN.energy_ratio(f, e, True) for _, _, e in ss]
    finally:
        f.close()
    return {"cycle": "V(2,2) bgs/rbgs", "plain": round(float(np.mean(plain)), 4),
            "learned": round(float(np.mean(learned)), 4), "samples": samples}


def run_reference(args, dist: Dist):
    if dist.rank != 0:
        return
    As, Ps, b, bs, gen_s, _ = generate(args)
    threads = os.cpu_count() or 1
    ref_nat, _ = reference_iterations(args)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.set_threads(threads)
    if args.warmup > 0:
        O.fcgmg_solve(As, Ps, b, bs, maxit=args.warmup, tol=0.0)
    x, hist, it, rc = O.fcgmg_solve(As, Ps, b, bs, maxit=args.steps, tol=0.0)
    setup_s, iter_s = O.last_timing()
    per_it = iter_s / max(it, 1)
    its = ref_nat if ref_nat else 35
    value = per_it * its
    n0 = As[0].shape[0]
    line = {
        "metric": METRIC, "value": round(value, 4), "unit": "s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(per_it * 1e3, 2), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
        "data": (f"synthetic: the reference's own {args.n}^{args.dim} HHO system ({args.coefficient} coefficient), "
                 "generated on the host"),
        "config": workload_config(args, n0, len(As)),
        "parallelism": f"{threads} host threads",
        "method": {"name": "plain FP64 FCG(1) + V(1,1) bgs/rbgs (the reference's method, natural block-GS order)",
                   "krylov": "FCG(1)", "cycle": "V(1,1) bgs/rbgs", "vcycle_precision": "fp64",
                   "coarsest": "FP64 direct solve"},
        "cpu_baseline": {"value": round(value, 4), "unit": "s", "cores": threads, "kind": "port",
                         "sample": (f"{it} FCG(1)+V(1,1) iterations (one per step) of the {n0}-unknown solve by the "
                                    f"oracle restatement of the reference (natural block-GS order, OpenMP "
                                    f"row-parallel products), {per_it:.3f} s/iteration x {its} reference iterations")},
        "e2e": {"value": round(value, 4), "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "setup_s": {"hierarchy_generation": round(gen_s, 2), "oracle_setup": round(setup_s, 2)},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus != world:
        # one process per GPU: N > 1 runs under torchrun (WORLD_SIZE = N), never N in one process
        sys.exit(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}; run N > 1 as "
                 f"python -m torch.distributed.run --nproc-per-node {args.gpus} bench.py --gpus {args.gpus}")
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
