"""Parity of the CUDA path (libfhg through its C ABI) with the reference and the oracle.

Solve level: iteration counts exact, normalised residual histories within 1e-10 relative per
iteration (absolute floor 1e-13), solutions within 1e-10 relative L2, against the reference's
own classes run on the colour-permuted hierarchy (tests/golden/). Kernel level: every operator
of every level against the oracle. Integer work (colour permutation): bit-exact.
"""
import importlib
import os

import numpy as np
import pytest
import scipy.sparse as sp

import oracle as O
from _golden import FULL_CASES, Case, available
from test_oracle import HIST_ATOL, X_RTOL, check_bj23_history, hist_close

pytestmark = pytest.mark.gpu

B = importlib.import_module("fhhos4_gb300.build")


@pytest.fixture(scope="session", autouse=True)
def built_library():
    if not os.path.exists(B.LIB):
        B.build()
    from fhhos4_gb300 import _native as N
    N.load()


@pytest.fixture(scope="module", params=available(FULL_CASES))
def case(request):
    return Case(request.param)


def S():
    from fhhos4_gb300 import solver
    return solver


def scalar_perm(perm, bs):
    return (np.asarray(perm)[:, None] * bs + np.arange(bs)[None, :]).ravel()


def true_rel_residual(A, b, x):
    return np.linalg.norm(b - A @ x) / np.linalg.norm(b)


# ---------------------------------------------------------------------------- solves
@pytest.mark.parametrize("graphs", [True, False])
def test_fcg_mg_matches_reference_colour_order(case, graphs):
    solver = S().fcg_mg(case.As, case.Ps, case.bs, use_graphs=graphs)
    hist = []
    solver.OnIterationEnd = lambda r: hist.append(r.NormalizedResidualNorm)
    x = solver.Solve(case.b)
    ref = case["hist_colour"]
    assert solver.IterationCount == len(ref) - 1
    assert hist_close(hist, ref), (np.asarray(hist), ref)
    xc = case["x_colour"]
    sp_ = scalar_perm(case.perms[0], case.bs)
    assert np.linalg.norm(x[sp_] - xc) / np.linalg.norm(xc) < X_RTOL
    # the colour permutation the GPU used is the oracle's, bit for bit
    ctx = solver.Context()
    for l in range(case.levels - 1):
        nb = case.As[l].shape[0] // case.bs
        assert np.array_equal(ctx.permutation(l, nb), case.perms[l])


def test_fcg_mg_on_the_permuted_hierarchy_is_the_reference_run(case):
    # The exact inputs the reference harness received; greedy colouring of a colour-grouped
    # matrix is the identity, so the GPU sweeps the rows in the same order.
    Ac, Pc, bc = O.permute_hierarchy(case.As, case.Ps, case.b, case.bs, case.perms)
    solver = S().fcg_mg(Ac, Pc, case.bs)
    x = solver.Solve(bc)
    ref = case["hist_colour"]
    assert solver.IterationCount == len(ref) - 1
    assert hist_close(solver.History, ref)
    assert np.linalg.norm(x - case["x_colour"]) / np.linalg.norm(case["x_colour"]) < X_RTOL
    ctx = solver.Context()
    for l in range(case.levels - 1):
        nb = Ac[l].shape[0] // case.bs
        assert np.array_equal(ctx.permutation(l, nb), np.arange(nb))


def test_pcg_mg_matches_reference(case):
    solver = S().fcg_mg(case.As, case.Ps, case.bs, krylov="cg")
    x = solver.Solve(case.b)
    ref = case["hist_cg"]
    assert solver.IterationCount == len(ref) - 1
    assert hist_close(solver.History, ref)
    sp_ = scalar_perm(case.perms[0], case.bs)
    assert np.linalg.norm(x[sp_] - case["x_cg"]) / np.linalg.norm(case["x_cg"]) < X_RTOL


@pytest.mark.parametrize("variant,pre,post,cycle", [("w", "bgs", "rbgs", "W"), ("sbgs", "sbgs", "sbgs", "V"),
                                                   ("abgs", "abgs", "rabgs", "V"), ("k", "bgs", "rbgs", "K")])
def test_cycles_and_smoothers_match_reference(case, variant, pre, post, cycle):
    solver = S().fcg_mg(case.As, case.Ps, case.bs, pre=pre, post=post, cycle=cycle)
    x = solver.Solve(case.b)
    ref = case[f"hist_{variant}"]
    assert solver.IterationCount == len(ref) - 1
    assert hist_close(solver.History, ref)
    sp_ = scalar_perm(case.perms[0], case.bs)
    xr = case[f"x_{variant}"]
    assert np.linalg.norm(x[sp_] - xr) / np.linalg.norm(xr) < X_RTOL


@pytest.mark.parametrize("variant,pre,post", [("sor", "bsor", "rbsor"), ("ssor", "sbsor", "sbsor")])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_block_sor_matches_reference(case, variant, pre, post, precision):
    """Block SOR, relaxation 1.2 (BlockSOR.h:99-227): FP64 at the reference's bar; the FP32 V-cycle
    reaches the FP64 tolerance with the FP64 true residual."""
    omega = float(case["sor_omega"])
    solver = S().fcg_mg(case.As, case.Ps, case.bs, pre=pre, post=post, omega=omega, precision=precision)
    x = solver.Solve(case.b)
    ref = case[f"hist_{variant}"]
    if precision == "fp32":
        assert solver.History[-1] < 1e-8 and true_rel_residual(case.As[0], case.b, x) < 1e-8 * (1 + 1e-6)
        assert solver.IterationCount <= len(ref) - 1 + 3
        return
    assert solver.IterationCount == len(ref) - 1
    assert hist_close(solver.History, ref)
    sp_ = scalar_perm(case.perms[0], case.bs)
    xr = case[f"x_{variant}"]
    assert np.linalg.norm(x[sp_] - xr) / np.linalg.norm(xr) < X_RTOL


def test_hybrid_codes_run_the_parallel_sweeps(case):
    """"hbgs"/"hrbgs" (the reference's chunk-parallel sweeps, schedule-dependent) run as the
    multicolour sweeps: the same solve as bgs/rbgs."""
    a = S().fcg_mg(case.As, case.Ps, case.bs, pre="hbgs", post="hrbgs")
    b = S().fcg_mg(case.As, case.Ps, case.bs)
    xa, xb = a.Solve(case.b), b.Solve(case.b)
    assert a.IterationCount == b.IterationCount and np.array_equal(xa, xb)


@pytest.mark.parametrize("nu,coarse_nu", [((1, 1), (2, 2)), ((2, 2), (4, 3))])
def test_coarse_smoothing_counts_match_the_oracle(case, nu, coarse_nu):
    """Smoothing counts per level (levels >= 1 apart from level 0; no counterpart in the reference)
    against the oracle extended the same way, on the colour-permuted hierarchy: exact iterations,
    histories within the parity tolerance."""
    Ac, Pc, bc = O.permute_hierarchy(case.As, case.Ps, case.b, case.bs, case.perms)
    _, h_o, it_o, st = O.fcgmg_solve(Ac, Pc, bc, case.bs, pre_iterations=nu[0], post_iterations=nu[1],
                                     coarse_iterations=coarse_nu)
    assert st == 0
    solver = S().fcg_mg(Ac, Pc, case.bs, nu=nu, coarse_nu=coarse_nu)
    solver.Solve(bc)
    assert solver.IterationCount == it_o
    assert hist_close(solver.History, h_o)
    # the setter on a context set up without coarse counts gives the same run
    from fhhos4_gb300 import _native as N
    plain = S().fcg_mg(Ac, Pc, case.bs, nu=nu)   # keeps its context alive
    ctx = plain.Context()
    ctx.set_coarse_smoothing(*coarse_nu)
    rc, x, hist, info = ctx.solve(bc, 200)
    assert rc == N.FHG_OK and info.iterations == it_o
    assert hist_close(hist[: it_o + 1], h_o)


def test_kcycle_with_fp32_vcycle_reaches_fp64_tolerance(case):
    """K-cycle with FP32 cycles inside the FP64 FCG: the FP64 true residual meets 1e-8 within a few
    iterations of the reference's FP64 K-cycle."""
    solver = S().fcg_mg(case.As, case.Ps, case.bs, cycle="K", precision="fp32")
    x = solver.Solve(case.b)
    ref = case["hist_k"]
    assert abs(solver.IterationCount - (len(ref) - 1)) <= 3
    assert true_rel_residual(case.As[0], case.b, x) < 1e-8 * (1 + 1e-6)


def test_block_jacobi_smoother_matches_reference(case):
    solver = S().fcg_mg(case.As, case.Ps, case.bs, pre="bj23", post="bj23")
    solver.Solve(case.b)
    check_bj23_history(solver.History, np.asarray(case["hist_bj23"]))


def test_solves_are_bitwise_reproducible(case):
    solver = S().fcg_mg(case.As, case.Ps, case.bs)
    x1 = solver.Solve(case.b)
    h1 = solver.History.copy()
    x2 = solver.Solve(case.b)
    assert np.array_equal(x1, x2) and np.array_equal(h1, solver.History)


@pytest.mark.parametrize("outer_split", [True, False])
def test_fp32_vcycle_reaches_fp64_tolerance(case, outer_split):
    ref_iters = len(case["hist_colour"]) - 1
    solver = S().fcg_mg(case.As, case.Ps, case.bs, precision="fp32", outer_split=outer_split)
    x = solver.Solve(case.b)
    assert solver.History[-1] < 1e-8
    assert solver.IterationCount <= ref_iters + 3
    assert true_rel_residual(case.As[0], case.b, x) < 5e-8
    xr = case["x_natural"]
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-6


def test_slot_major_gs_solve_tracks_row_major(case):
    """The FP32 fast cycle with slot-major GS sweeps: the same arithmetic as the row-major sweeps up
    to FP32 summation order, so the same iterations within one and the FP64 tolerance."""
    kw = dict(precision="fp32", nu=(3, 3), coarse_nu=(4, 4))
    a = S().fcg_mg(case.As, case.Ps, case.bs, gs_layout="row", **kw)
    a.Solve(case.b)
    b = S().fcg_mg(case.As, case.Ps, case.bs, gs_layout="slot", **kw)
    xb = b.Solve(case.b)
    assert abs(a.IterationCount - b.IterationCount) <= 1
    assert b.History[-1] < 1e-8
    assert true_rel_residual(case.As[0], case.b, xb) < 5e-8


def test_double_fp32_outer_product_tracks_fp64(case):
    # The double-FP32 outer product (FP64-class accuracy, ~1e-14 relative per product) changes
    # the FP32-V-cycle solve at the FP32 rounding level of the V-cycle only: same iteration count
    # within one, histories within 1e-5 relative, same FP64 true residual tolerance.
    a = S().fcg_mg(case.As, case.Ps, case.bs, precision="fp32", outer_split=True)
    xa = a.Solve(case.b)
    b = S().fcg_mg(case.As, case.Ps, case.bs, precision="fp32", outer_split=False)
    b.Solve(case.b)
    assert abs(a.IterationCount - b.IterationCount) <= 1
    m = min(len(a.History), len(b.History))
    assert np.all(np.abs(a.History[:m] - b.History[:m]) <= 1e-5 * b.History[:m] + 1e-13)
    assert true_rel_residual(case.As[0], case.b, xa) < 5e-8
    # the product itself: double-FP32 against FP64 on the outer operator
    from fhhos4_gb300 import _native as N
    rng = np.random.default_rng(3)
    d = rng.standard_normal(case.As[0].shape[0])
    y64 = a.Context().apply(0, N.OP_SYM_SPMV, d, None, len(d))
    y_ref = O.spmv_sym_lower(case.As[0], d)
    assert np.linalg.norm(y64 - y_ref) <= 1e-13 * np.linalg.norm(y_ref)


def test_autotuned_lanes_give_the_same_solve(case):
    solver = S().fcg_mg(case.As, case.Ps, case.bs, autotune=True)
    solver.Solve(case.b)
    ref = case["hist_colour"]
    assert solver.IterationCount == len(ref) - 1
    assert hist_close(solver.History, ref)


# ------------------------------------------------------- FP64-class V-cycle in FP32 pairs (df)
DF_VARIANTS = [("colour", "bgs", "rbgs", "V", None), ("w", "bgs", "rbgs", "W", None),
               ("sbgs", "sbgs", "sbgs", "V", None), ("abgs", "abgs", "rabgs", "V", None),
               ("k", "bgs", "rbgs", "K", None), ("sor", "bsor", "rbsor", "V", "sor_omega")]


@pytest.mark.parametrize("variant,pre,post,cycle,omega_key,layout",
                         [v + ("auto",) for v in DF_VARIANTS] + [DF_VARIANTS[0] + ("slot",)])
def test_df_vcycle_matches_reference(case, variant, pre, post, cycle, omega_key, layout):
    """The pair V-cycle (FHG_PREC_DF: operators, D^-1 and vectors as FP32 pairs, the outer FCG in pair
    arithmetic with FP64 x) at the reference's own bar: iteration counts exact, histories within
    1e-10, x within 1e-10 (row-major views, and slot-major sweeps and products)."""
    omega = float(case[omega_key]) if omega_key else 1.0
    solver = S().fcg_mg(case.As, case.Ps, case.bs, pre=pre, post=post, cycle=cycle, omega=omega, precision="df",
                        gs_layout=layout)
    x = solver.Solve(case.b)
    ref = case[f"hist_{variant}"]
    assert solver.IterationCount == len(ref) - 1
    # Absolute floor 2^6 times the FP64 one: pairs carry 47-48 bits, so a residual at the rounding
    # level of an exact coarse solve (one-iteration cases) sits 64 times higher than in FP64.
    h, r = np.asarray(solver.History), np.asarray(ref)
    assert np.all(np.abs(h - r) <= 1e-10 * np.abs(r) + 64 * HIST_ATOL), (h, r)
    sp_ = scalar_perm(case.perms[0], case.bs)
    xr = case[f"x_{variant}"]
    assert np.linalg.norm(x[sp_] - xr) / np.linalg.norm(xr) < X_RTOL


@pytest.mark.parametrize("precision,cycle,pre,post", [("fp32", "V", "bgs", "rbgs"), ("df", "V", "bgs", "rbgs"),
                                                       ("df", "W", "sbgs", "sbgs"), ("fp32", "W", "bgs", "rbgs"),
                                                       ("fp32", "V", "bsor", "rbsor")])
def test_fused_coarse_cycle_matches_launch_by_launch(case, precision, cycle, pre, post):
    """The coarse sub-cycle as one cluster launch (CTAs of 512 and of 1024 threads) against the same
    cycle launched phase by phase: the same arithmetic up to the summation order of a row, so FP64-class solves agree to 1e-10
    (iterations equal) and FP32 solves take the same iterations within one and reach the tolerance."""
    kw = dict(precision=precision, cycle=cycle, pre=pre, post=post, nu=(2, 2), coarse_nu=(3, 3),
              omega=float(case["sor_omega"]) if pre == "bsor" else 1.0)
    b = S().fcg_mg(case.As, case.Ps, case.bs, fused=False, **kw)
    assert b._ctx.fused_coarse_info(precision)[0] == -1
    for fused, threads in ((True, 512), ("wide", 1024)):
        a = S().fcg_mg(case.As, case.Ps, case.bs, fused=fused, **kw)
        first, ctas, nthreads = a._ctx.fused_coarse_info(precision)
        if len(case.As) >= 3:
            assert 1 <= first <= len(case.As) - 2 and ctas == 8 and nthreads == threads
        _check_fused_pair(case.As[0], case.b, a, b, precision)


def _check_fused_pair(A0, rhs, a, b, precision, rtol=1e-10):
    xa, xb = a.Solve(rhs), b.Solve(rhs)
    if precision == "df":
        assert a.IterationCount == b.IterationCount
        assert np.all(np.abs(a.History - b.History) <= rtol * np.abs(b.History) + 64 * HIST_ATOL)
        assert np.linalg.norm(xa - xb) <= rtol * np.linalg.norm(xb)
    else:
        assert abs(a.IterationCount - b.IterationCount) <= 1
        assert true_rel_residual(A0, rhs, xa) < 1e-8 * (1 + 1e-6)


@pytest.mark.parametrize("precision,cycle", [("fp32", "V"), ("df", "V"), ("df", "W")])
def test_fused_coarse_cycle_deep_hierarchy(precision, cycle):
    """A deep 2D hierarchy (n = 256, k = 3: six levels, Galerkin coarse operators, the largest
    problem of the batched workload), fused with CTAs of 512 and 1024 threads and chosen by timing:
    the same answers as launch by launch. The sub-cycle runs as a loop over levels with fixed stack use.
    Rows of the Galerkin operators hold about 40 blocks, summed by 16 lanes here and by the tuned
    launch shape there; with the coefficient contrast (1e3) FCG carries that reordering (a few units
    of 2^-47 per row in pairs) to 1e-10 of the history, so the FP64-class bar is 1e-8."""
    from fhhos4_gb300 import batch as BT
    bs, A0, Ps, b, levels = BT.generate(BT.ProblemSpec(256, 3, 4242))
    As = [A0]
    for P in Ps:
        As.append((P.T @ As[-1] @ P).tocsr())
    kw = dict(precision=precision, cycle=cycle, pre="bgs", post="rbgs", galerkin=True)
    b_ = S().fcg_mg(As, Ps, bs, fused=False, **kw)
    for fused, autotune in ((True, False), ("wide", False), (True, True)):
        a = S().fcg_mg(As, Ps, bs, fused=fused, autotune=autotune, **kw)
        first, ctas, threads = a._ctx.fused_coarse_info(precision)
        assert first == -1 or (1 <= first <= len(As) - 2 and ctas in (8, 16) and threads in (512, 1024))
        if not autotune:
            assert first >= 1 and threads == (1024 if fused == "wide" else 512)
        _check_fused_pair(A0, b, a, b_, precision, rtol=1e-8)


def _pairs(torch, v):
    """An FP64 vector as interleaved FP32 pairs (hi, lo) on the device."""
    hi = v.astype(np.float32)
    lo = (v - hi.astype(np.float64)).astype(np.float32)
    return torch.tensor(np.stack([hi, lo], axis=1), device="cuda")


def _unpair(t):
    a = t.cpu().numpy().astype(np.float64)
    return a[:, 0] + a[:, 1]


@pytest.mark.parametrize("layout", ["row", "slot"])
def test_df_operators_of_every_level(case, layout):
    """Every pair operator of every level (row- or slot-major padded views) against the oracle in
    FP64, to FP64-class accuracy."""
    torch = pytest.importorskip("torch")
    from fhhos4_gb300 import _native as N
    solver = S().fcg_mg(case.As, case.Ps, case.bs, precision="df", gs_layout=layout)
    ctx = solver.Context()
    rng = np.random.default_rng(5)
    tol = 1e-12
    for l, A in enumerate(case.As):
        n = A.shape[0]
        s = scalar_perm(ctx.permutation(l, n // case.bs), case.bs)
        Ap = O.as_csr(A[s][:, s])
        x = rng.standard_normal(n)
        b = rng.standard_normal(n)
        xd, bd = _pairs(torch, x), _pairs(torch, b)
        out = torch.zeros_like(xd)
        scale = np.abs(A).max() * np.linalg.norm(x) + np.linalg.norm(b)
        ctx.apply_internal(l, N.OP_SPMV, "df", xd.data_ptr(), None, out.data_ptr())
        assert np.linalg.norm(_unpair(out) - O.spmv(Ap, x)) <= tol * scale, l
        ctx.apply_internal(l, N.OP_RESIDUAL, "df", xd.data_ptr(), bd.data_ptr(), out.data_ptr())
        assert np.linalg.norm(_unpair(out) - O.residual(Ap, b, x)) <= tol * scale, l
        if l < case.levels - 1:
            for op, backward in ((N.OP_GS_FORWARD, False), (N.OP_GS_BACKWARD, True)):
                ctx.apply_internal(l, op, "df", xd.data_ptr(), bd.data_ptr(), out.data_ptr())
                ref = O.block_gs(Ap, case.bs, b, x, backward=backward)
                assert np.linalg.norm(_unpair(out) - ref) <= 1e-11 * np.linalg.norm(ref), (l, op)
            ctx.apply_internal(l, N.OP_JACOBI, "df", xd.data_ptr(), bd.data_ptr(), out.data_ptr())
            ref = O.block_jacobi(Ap, case.bs, 1.0, b, x)
            assert np.linalg.norm(_unpair(out) - ref) <= 1e-11 * np.linalg.norm(ref), l
            sc = scalar_perm(ctx.permutation(l + 1, case.As[l + 1].shape[0] // case.bs), case.bs)
            Pp = O.as_csr(case.Ps[l][s][:, sc])
            nc = Pp.shape[1]
            rc = torch.zeros((nc, 2), dtype=torch.float32, device="cuda")
            ctx.apply_internal(l, N.OP_RESTRICT, "df", xd.data_ptr(), None, rc.data_ptr())
            ref = O.spmv(O.as_csr(Pp.T), x)
            assert np.linalg.norm(_unpair(rc) - ref) <= tol * np.abs(Pp).max() * np.linalg.norm(x) * 10, l
            e = rng.standard_normal(nc)
            ed = _pairs(torch, e)
            ctx.apply_internal(l, N.OP_PROLONG_ADD, "df", ed.data_ptr(), xd.data_ptr(), out.data_ptr())
            ref = x + O.spmv(Pp, e)
            assert np.linalg.norm(_unpair(out) - ref) <= tol * (np.linalg.norm(x) + np.abs(Pp).max() * np.linalg.norm(e)) * 10
        else:
            ctx.apply_internal(l, N.OP_COARSE_SOLVE, "df", bd.data_ptr(), None, out.data_ptr())
            ref = np.linalg.solve(Ap.toarray(), b)
            assert np.linalg.norm(_unpair(out) - ref) <= 1e-10 * np.linalg.norm(ref)


# ---------------------------------------------------------------------------- kernels
def _ctx(case):
    solver = S().fcg_mg(case.As, case.Ps, case.bs)
    return solver, solver.Context()


def test_operators_of_every_level(case):
    from fhhos4_gb300 import _native as N
    solver, ctx = _ctx(case)
    rng = np.random.default_rng(7)
    for l, A in enumerate(case.As):
        n = A.shape[0]
        x = rng.standard_normal(n)
        b = rng.standard_normal(n)
        scale = np.abs(A).max() * np.linalg.norm(x)
        y = ctx.apply(l, N.OP_SPMV, x, None, n)
        assert np.linalg.norm(y - O.spmv(A, x)) <= 1e-14 * scale * 10
        r = ctx.apply(l, N.OP_RESIDUAL, x, b, n)
        assert np.linalg.norm(r - O.residual(A, b, x)) <= 1e-14 * (scale + np.linalg.norm(b)) * 10
        if l < case.levels - 1:
            P = case.Ps[l]
            nc = P.shape[1]
            R = O.as_csr(P.T)
            rc = ctx.apply(l, N.OP_RESTRICT, x, None, nc)
            assert np.linalg.norm(rc - O.spmv(R, x)) <= 1e-13 * np.abs(P).max() * np.linalg.norm(x) * 10
            e = rng.standard_normal(nc)
            xp = ctx.apply(l, N.OP_PROLONG_ADD, e, x, n)
            assert np.linalg.norm(xp - (x + O.spmv(P, e))) <= 1e-13 * (np.linalg.norm(x) + np.abs(P).max() * np.linalg.norm(e)) * 10
            # smoothers: the GPU sweeps in colour order; the oracle sweeps the permuted matrix
            s = scalar_perm(ctx.permutation(l, n // case.bs), case.bs)
            Ap = O.as_csr(A[s][:, s])
            for op, backward in ((N.OP_GS_FORWARD, False), (N.OP_GS_BACKWARD, True)):
                g = ctx.apply(l, op, x, b, n)
                ref = np.empty(n)
                ref[s] = O.block_gs(Ap, case.bs, b[s], x[s], backward=backward)
                assert np.linalg.norm(g - ref) <= 1e-11 * np.linalg.norm(ref)
            j = ctx.apply(l, N.OP_JACOBI, x, b, n)
            assert np.linalg.norm(j - O.block_jacobi(A, case.bs, 1.0, b, x)) <= 1e-11 * np.linalg.norm(j)
        else:
            xs = ctx.apply(l, N.OP_COARSE_SOLVE, b, None, n)
            ref = np.linalg.solve(A.toarray(), b)
            assert np.linalg.norm(xs - ref) <= 1e-10 * np.linalg.norm(ref)
    A0 = case.As[0]
    x = rng.standard_normal(A0.shape[0])
    ys = ctx.apply(0, N.OP_SYM_SPMV, x, None, A0.shape[0])
    assert np.linalg.norm(ys - O.spmv_sym_lower(A0, x)) <= 1e-13 * np.abs(A0).max() * np.linalg.norm(x) * 10


@pytest.mark.parametrize("layout", ["row", "slot"])
def test_fp32_smoothers_of_every_level(case, layout):
    """FP32 GS sweeps (on the padded off-diagonal view where setup built one, row- or slot-major), the
    residual product (on the same layout's view of A) and block Jacobi on every smoothed level against
    the FP64 oracle in colour order, to FP32 accuracy."""
    torch = pytest.importorskip("torch")
    from fhhos4_gb300 import _native as N
    solver = S().fcg_mg(case.As, case.Ps, case.bs, precision="fp32", gs_layout=layout)
    ctx = solver.Context()
    rng = np.random.default_rng(11)
    for l in range(case.levels - 1):
        A = case.As[l]
        n = A.shape[0]
        s = scalar_perm(ctx.permutation(l, n // case.bs), case.bs)
        Ap = O.as_csr(A[s][:, s])
        x = rng.standard_normal(n).astype(np.float32).astype(np.float64)
        b = rng.standard_normal(n).astype(np.float32).astype(np.float64)
        xd = torch.tensor(x, dtype=torch.float32, device="cuda")
        bd = torch.tensor(b, dtype=torch.float32, device="cuda")
        out = torch.empty_like(xd)
        for op, backward in ((N.OP_GS_FORWARD, False), (N.OP_GS_BACKWARD, True)):
            ctx.apply_internal(l, op, "fp32", xd.data_ptr(), bd.data_ptr(), out.data_ptr())
            ref = O.block_gs(Ap, case.bs, b, x, backward=backward)
            g = out.cpu().numpy().astype(np.float64)
            assert np.linalg.norm(g - ref) <= 2e-4 * np.linalg.norm(ref), (l, op)
        # products with A on the same layout's view
        scale = np.abs(A).max() * np.linalg.norm(x) + np.linalg.norm(b)
        ctx.apply_internal(l, N.OP_RESIDUAL, "fp32", xd.data_ptr(), bd.data_ptr(), out.data_ptr())
        g = out.cpu().numpy().astype(np.float64)
        assert np.linalg.norm(g - O.residual(Ap, b, x)) <= 1e-5 * scale, l
        ctx.apply_internal(l, N.OP_JACOBI, "fp32", xd.data_ptr(), bd.data_ptr(), out.data_ptr())
        ref = O.block_jacobi(Ap, case.bs, 1.0, b, x)
        g = out.cpu().numpy().astype(np.float64)
        assert np.linalg.norm(g - ref) <= 2e-4 * np.linalg.norm(ref), l


def test_kernel_launches_are_counted(case):
    solver, ctx = _ctx(case)
    before = ctx.kernel_launches()
    solver.Solve(case.b)
    assert ctx.kernel_launches() > before + solver.IterationCount


# ---------------------------------------------------------------------------- errors
def _tiny():
    c = Case("tet3d_n4_k1")
    return c


def test_nan_rhs_reports_the_reference_message():
    from fhhos4_gb300 import _native as N
    c = _tiny()
    solver = S().fcg_mg(c.As, c.Ps, c.bs)
    b = c.b.copy()
    b[5] = np.nan
    with pytest.raises(N.FhgError) as ei:
        solver.Solve(b)
    assert ei.value.code in (N.FHG_ERR_NAN, N.FHG_ERR_DIVERGED)


def test_singular_diagonal_block_is_rejected():
    from fhhos4_gb300 import _native as N
    c = _tiny()
    A = c.As[0].tolil()
    A[0, :] = 0.0
    A[:, 0] = 0.0
    A = sp.csr_matrix(A)
    A.eliminate_zeros()
    with pytest.raises(N.FhgError) as ei:
        S().fcg_mg([A] + c.As[1:], c.Ps, c.bs)
    assert ei.value.code == N.FHG_ERR_SINGULAR_BLOCK


def test_fp64_setup_after_fp32_drops_the_fp32_operators():
    """A context set up again in FP64 keeps no FP32 operator of its earlier FP32 setup: switching
    its V-cycle to FP32 is refused (the FP32 data were freed with the first setup)."""
    from fhhos4_gb300 import _native as N
    c = _tiny()
    ctx = N.Context(0)
    for l, A in enumerate(c.As):
        ctx.set_level(l, c.bs, A)
    for l, P in enumerate(c.Ps):
        ctx.set_prolongation(l, P)
    o = N.default_options()
    o.vcycle_precision = N.PRECISION["fp32"]
    ctx.setup(len(c.As), o)
    ctx.set_vcycle_precision("fp32")
    o.vcycle_precision = N.PRECISION["fp64"]
    ctx.setup(len(c.As), o)
    with pytest.raises(N.FhgError) as ei:
        ctx.set_vcycle_precision("fp32")
    assert ei.value.code == N.FHG_ERR_NOT_READY
    rc, x, hist, info = ctx.solve(c.b, 200)
    assert rc == N.FHG_OK and info.normalized_residual < 1e-8
    ctx.close()


def test_invalid_inputs_are_rejected():
    from fhhos4_gb300 import _native as N
    c = _tiny()
    ctx = N.Context(0)
    with pytest.raises(N.FhgError) as ei:
        ctx.set_level(0, 5, c.As[0])
    assert ei.value.code == N.FHG_ERR_UNSUPPORTED
    with pytest.raises(N.FhgError) as ei:
        ctx.setup(2, N.default_options())
    assert ei.value.code == N.FHG_ERR_INVALID_ARG
    ctx.set_level(0, c.bs, c.As[0])
    ctx.set_level(1, c.bs, c.As[1])
    with pytest.raises(N.FhgError):
        ctx.setup(2, N.default_options())          # P_0 missing
    ctx.set_prolongation(0, c.Ps[0])
    o = N.default_options()
    o.max_coarse_rows = 10
    with pytest.raises(N.FhgError) as ei:
        ctx.setup(2, o)
    assert ei.value.code == N.FHG_ERR_TOO_LARGE
    rc, x, hist, info = ctx.solve(c.b, 10)
    assert rc == N.FHG_ERR_NOT_READY
    ctx.setup(2, N.default_options())
    rc, x, hist, info = ctx.solve(c.b, 200)
    assert rc == N.FHG_OK and info.iterations > 0
    bad = sp.csr_matrix(c.As[0])
    bad.indices = bad.indices.copy()
    bad.indices[0] = bad.shape[0] + 3
    with pytest.raises(N.FhgError) as ei:
        ctx.set_level(0, c.bs, bad)
    assert ei.value.code == N.FHG_ERR_INVALID_ARG
    ctx.close()
