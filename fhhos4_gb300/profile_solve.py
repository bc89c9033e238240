"""Solve one HHO problem a few times inside an NVTX range, for profilers.

    python -m fhhos4_gb300.profile_solve --n 64 --solves 1 [--method learned|fast|plain]

Setup (hierarchy generation, upload, autotuning) and warm-up solves run outside the range
"solve"; `ncu --nvtx --nvtx-include "solve/" ...` then captures the launches of the timed solves
only. `--step` instead applies one level-0 operator inside the range (the learned step, a forward
GS sweep, the double-FP32 outer product, the SpMV in pair or native FP64 arithmetic, the FP32
restriction or prolongation). `--p-multigrid ch|mg` instead times FCG with the p-multigrid
preconditioner against FCG with the h-multigrid one at the same degree (pair and FP32 V-cycles,
default launch shapes) and prints one JSON line.
"""
from __future__ import annotations

import argparse
import json


def p_multigrid_timing(a):
    """FCG(1) with the p-multigrid preconditioner of "-s fcgp_mg -cs <a.p_multigrid>" against FCG(1)
    with the h-multigrid one (V(1,1) bgs/rbgs) on the same degree-k problem: the library's solve time
    of the faster of two solves after one untimed, iterations and the FP64 true residual."""
    import numpy as np
    from . import hho
    from . import solver as S
    As, Ps, b, bss, cnu = hho.generate_p(a.dim, a.n, a.k, a.p_multigrid)
    H = hho.Hierarchy(a.dim, a.n, a.k)
    Ah, Ph = [H.A(l) for l in range(H.levels)], [H.P(l) for l in range(H.levels - 1)]
    H.close()
    out = {"workload": f"{a.dim}D n={a.n} k={a.k}", "unknowns": As[0].shape[0],
           "p_mg": {"block_sizes": bss, "levels": [A.shape[0] for A in As], "coarse_solver": a.p_multigrid,
                    "coarse_nu": list(cnu)},
           "h_mg": {"levels": [A.shape[0] for A in Ah]}}
    for name, (AA, PP, bb, cn) in (("p_mg", (As, Ps, bss, cnu)), ("h_mg", (Ah, Ph, bss[0], (-1, -1)))):
        for prec in ("df", "fp32"):
            s = S.fcg_mg(AA, PP, bb, coarse_nu=cn, precision=prec)
            s.Solve(b)
            ms = []
            for _ in range(2):
                x = s.Solve(b)
                ms.append(s.SolveTimeMs)
            out[name][prec] = {"ms": round(min(ms), 3), "iterations": s.IterationCount,
                               "true_rel_residual": float(np.linalg.norm(b - As[0] @ x) / np.linalg.norm(b))}
            s.Context().close()
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dim", type=int, default=3)
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--k", type=int, default=1)
    ap.add_argument("--method", choices=["learned", "fast", "plain"], default="learned")
    ap.add_argument("--nu", default="2,2")
    ap.add_argument("--solves", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--autotune", type=int, default=1, help="0: default launch shapes (comparable across runs)")
    ap.add_argument("--coarse-nu", default="", help="pre,post smoothing steps on levels >= 1 (default: --nu)")
    ap.add_argument("--levels", type=int, default=0, help="use the first N levels (the last one solved directly)")
    ap.add_argument("--weights", default="", help="learned-step network (default: the committed one)")
    ap.add_argument("--gs-layout", default="auto", choices=["auto", "row", "slot"], help="FP32 GS sweep layout")
    ap.add_argument("--p-multigrid", default="", choices=["", "ch", "mg"],
                    help="compare FCG + p-multigrid (this coarse solver) with FCG + h-multigrid at --k")
    ap.add_argument("--step", choices=["", "learned_tcgen05", "learned_mma_sync", "gs_fp32", "outer_df", "spmv_df",
                                       "spmv_fp64", "restrict_fp32", "prolong_fp32"], default="")
    a = ap.parse_args()
    if a.p_multigrid:
        p_multigrid_timing(a)
        return

    import torch
    from . import _native as N
    from . import hho
    from . import learned as LN

    H = hho.Hierarchy(a.dim, a.n, a.k)
    As = [H.A(l) for l in range(H.levels)]
    Ps = [H.P(l) for l in range(H.levels - 1)]
    b, bs = H.b(), H.block_size
    ctx = N.Context(0)
    for l, A in enumerate(As):
        ctx.set_level(l, bs, A)
    for l, P in enumerate(Ps):
        ctx.set_prolongation(l, P)
    ctx.set_face_tensors(H.face_tensors(0))
    H.close()
    nlev = a.levels if a.levels > 0 else len(As)
    o = N.default_options()
    o.vcycle_precision = N.PRECISION["fp32"]
    o.extra_precisions = 1 << N.PRECISION["df"]   # the FP64-class pair copies as well
    o.autotune = a.autotune
    o.gs_layout = N.GS_LAYOUT[a.gs_layout]
    ctx.setup(nlev, o)
    npre, npost = (int(v) for v in a.nu.split(","))
    params = LN.load_params(a.weights or LN.DEFAULT_WEIGHTS)[0]
    if a.method == "plain":
        ctx.set_cycle("bgs", "rbgs", 1, 1, 1)
        ctx.set_vcycle_precision("fp64")
    else:
        ctx.set_cycle("bgs", "rbgs", npre, npost, 1)
        if a.coarse_nu:
            ctx.set_coarse_smoothing(*(int(v) for v in a.coarse_nu.split(",")))
        if a.method == "learned" and bs <= 4:
            ctx.set_learned(params, "fallback")
    bd = torch.from_numpy(b).cuda()
    xd = torch.empty_like(bd)
    torch.cuda.synchronize()
    out = {}
    if a.step:
        op, prec = {"learned_tcgen05": (N.OP_LEARNED_STEP, "fp32"), "learned_mma_sync": (N.OP_LEARNED_STEP, "fp32"),
                    "gs_fp32": (N.OP_GS_FORWARD, "fp32"), "outer_df": (N.OP_SYM_SPMV, "fp32"),
                    "spmv_df": (N.OP_SPMV, "df"), "spmv_fp64": (N.OP_SPMV, "fp64"),
                    "restrict_fp32": (N.OP_RESTRICT, "fp32"), "prolong_fp32": (N.OP_PROLONG_ADD, "fp32")}[a.step]
        if a.step.startswith("learned"):
            ctx.set_learned(params, "always", kernel=a.step.split("_", 1)[1])
        ctx.time_op(0, op, prec, warmup=a.warmup, reps=1)
        torch.cuda.nvtx.range_push("solve")
        out["ms"] = ctx.time_op(0, op, prec, warmup=0, reps=a.solves)
        torch.cuda.nvtx.range_pop()
    else:
        for _ in range(a.warmup):
            ctx.solve_device(bd.data_ptr(), xd.data_ptr(), 200)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("solve")
        for _ in range(a.solves):
            rc, hist, info = ctx.solve_device(bd.data_ptr(), xd.data_ptr(), 200)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        out = {"rc": rc, "iterations": info.iterations, "ms": info.solve_ms,
               "learned_iterations": info.learned_iterations}
    print(json.dumps(out), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
