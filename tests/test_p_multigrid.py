"""p-multigrid (src/Solver/Multigrid/MultigridForHHO/P_MultigridForHHO.h): levels of decreasing face
degree on the fine mesh joined by the natural injection, as "-s fcg -p p_mg" builds them, with the
coarse solvers "ch" (direct, on the lowest degree) and "mg" (one h-multigrid cycle on it, no
pre-smoothing and 3 (2D) or 6 (3D) post-smoothing steps, SolverFactory.h:289-309).

The fixtures (tests/golden/p_*.npz, make_golden.py --p-multigrid) hold the reference's own runs of
that path: its histories and solutions in its natural order, the block size of every level, and
A_l v_l, P_l v_l for seeded v_l. CPU: the generator's p-hierarchy against them, and the oracle on it
against the reference's histories. GPU: the CUDA path in the reference's order against the
reference itself, in colour order against the oracle (FP64, pairs, FP32, Galerkin), and the
injection transfers against P and P^T.
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp

import oracle as O
from _golden import GOLDEN
from test_oracle import HIST_ATOL, X_RTOL, hist_close

from fhhos4_gb300 import hho

P_CASES = [n for n in ("p_tri2d_n16_k3", "p_tet3d_n4_k2") if os.path.exists(os.path.join(GOLDEN, n + ".npz"))]
# b on tetrahedra: the reference's source quadrature (degree 8) against this generator's exact one
B_TOL = {2: 1e-13, 3: 1e-7}


class PCase:
    def __init__(self, name):
        self.name = name
        self.z = np.load(os.path.join(GOLDEN, name + ".npz"))
        self.dim, self.n, self.k = int(self.z["dim"]), int(self.z["n"]), int(self.z["k"])

    def __getitem__(self, key):
        return self.z[key]


def probe_vector(l, n):
    return np.random.default_rng(1000 + l).standard_normal(n)


@pytest.fixture(scope="module", params=P_CASES)
def case(request):
    return PCase(request.param)


@pytest.fixture(scope="module")
def hierarchies(case):
    """The generator's p-hierarchy for both coarse solvers: cs -> (As, Ps, b, block_sizes, coarse_nu)."""
    return {cs: hho.generate_p(case.dim, case.n, case.k, cs) for cs in ("ch", "mg")}


# ------------------------------------------------------------------------------------------ CPU
def test_p_degrees_follow_the_reference_rule():
    big = 10 ** 6
    assert hho.p_degrees(2, 3, big) == [3, 1]                        # Minus2, CoarsePolyDegree 1
    assert hho.p_degrees(2, 4, big) == [4, 2, 1]
    assert hho.p_degrees(2, 3, big, "minus1") == [3, 2, 1]
    assert hho.p_degrees(2, 5, big, "divide_by_2") == [5, 2, 1]
    assert hho.p_degrees(2, 5, big, "direct_to_low") == [5, 1]
    assert hho.p_degrees(2, 3, 10) == [3]                             # already at most 1000 unknowns
    with pytest.raises(ValueError, match="polynomial degree"):
        hho.p_degrees(2, 1, big)


def test_generate_p_refuses_what_the_cycle_cannot_express():
    """With the h-multigrid coarse solver the composite hierarchy smooths every level below the
    finest with the coarse solver's counts: that is the reference's cycle only with exactly two
    p-levels."""
    with pytest.raises(NotImplementedError, match="smoothing counts"):
        hho.generate_p(2, 16, 3, "mg", strategy="minus1")          # degrees 3, 2, 1
    with pytest.raises(NotImplementedError, match="lowest-degree"):
        hho.generate_p(2, 4, 3, "mg")                              # already at most 1000 unknowns
    with pytest.raises(ValueError):
        hho.generate_p(2, 16, 3, "lu")
    As, Ps, b, bss, cnu = hho.generate_p(2, 16, 3, "ch", strategy="minus1")
    assert bss == [4, 3, 2] and cnu == (-1, -1) and len(Ps) == 2


def test_natural_injection_structure():
    P = hho.natural_injection(5, 6, 3)
    assert P.shape == (30, 15) and P.nnz == 15 and np.all(P.data == 1.0)
    e = np.arange(15.0)
    assert np.array_equal((P @ e).reshape(5, 6)[:, :3], e.reshape(5, 3))
    assert np.all((P @ e).reshape(5, 6)[:, 3:] == 0)


def test_generated_p_hierarchy_matches_reference(case, hierarchies):
    As, Ps, b, bss, cnu = hierarchies["mg"]
    assert bss == [int(v) for v in case["block_sizes"]]
    assert len(As) == int(case["levels_mg"]) and len(hierarchies["ch"][0]) == int(case["levels_ch"])
    assert cnu == (0, 3 if case.dim == 2 else 6)
    for l, A in enumerate(As):
        # (stored-entry counts differ where one assembly keeps a rounding-level entry the other drops)
        assert A.shape == tuple(case[f"A{l}_shape"]), l
        ref = case[f"Av{l}"]
        assert np.abs(A @ probe_vector(l, A.shape[0]) - ref).max() <= 1e-12 * np.abs(ref).max(), l
    for l, P in enumerate(Ps):
        assert P.shape == tuple(case[f"P{l}_shape"]), l
        ref = case[f"Pv{l}"]
        got = P @ probe_vector(100 + l, P.shape[1])
        if l < int(case["p_levels"]) - 1:
            # the natural injection, bit for bit
            assert P.nnz == int(case[f"P{l}_nnz"]) and np.array_equal(got, ref), l
        else:
            assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), l
    assert np.linalg.norm(b - case["b"]) <= B_TOL[case.dim] * np.linalg.norm(case["b"])


@pytest.mark.parametrize("cs", ["ch", "mg"])
def test_oracle_p_multigrid_matches_reference(case, hierarchies, cs):
    """The oracle's cycle over the p-hierarchy (per-level block sizes; with "mg" the levels below the
    lowest degree smoothed V(0, 3/6)) reproduces the reference's own FCG + p_mg history. The
    reference's b is used, so only the operators' rounding separates the two."""
    As, Ps, b, bss, cnu = hierarchies[cs]
    x, hist, it, rc = O.fcgmg_solve(As, Ps, case["b"], bss, coarse_iterations=cnu)
    ref = case[f"hist_{cs}"]
    assert rc == 0 and it == len(ref) - 1
    assert hist_close(hist, ref), (hist, ref)
    xr = case[f"x_{cs}"]
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < X_RTOL


def test_oracle_three_p_levels_match_reference():
    """P_CoarsStgy Minus1 with the direct coarse solver: face degrees 3, 2, 1 (block sizes 4, 3, 2),
    two natural injections, every p-level smoothed V(1,1): the oracle against the reference's run."""
    z = np.load(os.path.join(GOLDEN, "p_tri2d_n16_k3.npz"))
    if "hist_ch_minus1" not in z.files:
        pytest.skip("fixture without the Minus1 case")
    As, Ps, b, bss, cnu = hho.generate_p(2, 16, 3, "ch", strategy="minus1")
    assert bss == [int(v) for v in z["block_sizes_ch_minus1"]]
    x, hist, it, rc = O.fcgmg_solve(As, Ps, z["b"], bss, coarse_iterations=cnu)
    ref = z["hist_ch_minus1"]
    assert rc == 0 and it == len(ref) - 1
    assert hist_close(hist, ref), (hist, ref)
    xr = z["x_ch_minus1"]
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < X_RTOL


# ------------------------------------------------------------------------------------------ GPU
def _solver():
    from fhhos4_gb300 import solver
    return solver


def _oracle_colour(As, Ps, b, bss, cnu, galerkin=False):
    """The oracle on the colour-permuted hierarchy (the order the GPU sweeps in)."""
    if galerkin:
        As = list(As[:1])
        for P in Ps:
            As.append(sp.csr_matrix(P.T @ As[-1] @ P))
    perms, _ = O.colour_perms(As, bss)
    Ac, Pc, bc = O.permute_hierarchy(As, Ps, b, bss, perms)
    x, hist, it, rc = O.fcgmg_solve(Ac, Pc, bc, bss, coarse_iterations=cnu)
    assert rc == 0
    sp0 = (np.asarray(perms[0])[:, None] * bss[0] + np.arange(bss[0])[None, :]).ravel()
    return x, hist, it, sp0, perms


@pytest.mark.gpu
@pytest.mark.parametrize("cs", ["ch", "mg"])
def test_gpu_p_multigrid_in_reference_order_is_the_reference(case, hierarchies, cs):
    """Colouring off (every block row its own colour: the reference's sequential block Gauss-Seidel),
    FP64: the GPU's FCG + p-multigrid against the reference's own run."""
    As, Ps, b, bss, cnu = hierarchies[cs]
    s = _solver().fcg_mg(As, Ps, bss, coarse_nu=cnu, precision="fp64", fused=False, colouring=False)
    x = s.Solve(case["b"])
    ref = case[f"hist_{cs}"]
    assert s.IterationCount == len(ref) - 1
    assert hist_close(s.History, ref), (s.History, ref)
    xr = case[f"x_{cs}"]
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < X_RTOL


@pytest.mark.gpu
@pytest.mark.parametrize("cs", ["ch", "mg"])
@pytest.mark.parametrize("precision", ["fp64", "df"])
def test_gpu_p_multigrid_colour_order_matches_oracle(case, hierarchies, cs, precision):
    As, Ps, b, bss, cnu = hierarchies[cs]
    xo, ho, it, sp0, perms = _oracle_colour(As, Ps, b, bss, cnu)
    s = _solver().fcg_mg(As, Ps, bss, coarse_nu=cnu, precision=precision)
    x = s.Solve(b)
    assert s.IterationCount == it
    h = np.asarray(s.History)
    floor = HIST_ATOL if precision == "fp64" else 64 * HIST_ATOL
    assert np.all(np.abs(h - ho) <= 1e-10 * np.abs(ho) + floor), (h, ho)
    assert np.linalg.norm(x[sp0] - xo) / np.linalg.norm(xo) < X_RTOL
    ctx = s.Context()
    for l in range(len(As) - 1):
        assert np.array_equal(ctx.permutation(l, As[l].shape[0] // bss[l]), perms[l]), l


@pytest.mark.gpu
@pytest.mark.parametrize("cs", ["ch", "mg"])
@pytest.mark.parametrize("fused", [True, False])
def test_gpu_p_multigrid_fp32_vcycle_reaches_tolerance(case, hierarchies, cs, fused):
    """The FP32 V-cycle inside the FCG (pair outer products): the FP64 true residual meets 1e-8 within
    two iterations of the FP64 method."""
    As, Ps, b, bss, cnu = hierarchies[cs]
    ref = _solver().fcg_mg(As, Ps, bss, coarse_nu=cnu, precision="fp64")
    ref.Solve(b)
    s = _solver().fcg_mg(As, Ps, bss, coarse_nu=cnu, precision="fp32", fused=fused)
    x = s.Solve(b)
    assert np.linalg.norm(b - As[0] @ x) / np.linalg.norm(b) < 1e-8 * (1 + 1e-6)
    assert s.IterationCount <= ref.IterationCount + 2


@pytest.mark.gpu
@pytest.mark.parametrize("cs", ["ch", "mg"])
def test_gpu_p_multigrid_galerkin(case, hierarchies, cs):
    """-g 1: every coarse operator P^T A P, on the injection level the leading block of every block
    (computed by the library), against the oracle on the same Galerkin hierarchy. On the 3D n = 4
    mesh the h-prolongation to n = 2 has rank 214 of its 216 columns, so the Galerkin operator below
    the lowest degree is singular (in h-multigrid alone as well): that case runs with "ch" only."""
    if cs == "mg" and case.dim == 3:
        pytest.skip("singular Galerkin coarse operator on the n = 2 tetrahedral mesh")
    As, Ps, b, bss, cnu = hierarchies[cs]
    xo, ho, it, sp0, _ = _oracle_colour(As, Ps, b, bss, cnu, galerkin=True)
    s = _solver().fcg_mg(As, Ps, bss, coarse_nu=cnu, precision="fp64", galerkin=True)
    x = s.Solve(b)
    assert s.IterationCount == it
    assert hist_close(s.History, ho), (s.History, ho)
    assert np.linalg.norm(x[sp0] - xo) / np.linalg.norm(xo) < X_RTOL


@pytest.mark.gpu
def test_gpu_injection_transfers_are_p_and_its_transpose(case, hierarchies):
    """The restriction and prolongation of the injection level, through the C ABI in the given
    numbering: P^T r and x + P e exactly (a copy and one addition per entry)."""
    from fhhos4_gb300 import _native as N
    As, Ps, b, bss, cnu = hierarchies["ch"]
    s = _solver().fcg_mg(As, Ps, bss, precision="fp64")
    ctx = s.Context()
    rng = np.random.default_rng(7)
    P = Ps[0]
    r = rng.standard_normal(P.shape[0])
    assert np.array_equal(ctx.apply(0, N.OP_RESTRICT, r, None, P.shape[1]), P.T @ r)
    e, x = rng.standard_normal(P.shape[1]), rng.standard_normal(P.shape[0])
    assert np.array_equal(ctx.apply(0, N.OP_PROLONG_ADD, e, x, P.shape[0]), x + P @ e)


@pytest.mark.gpu
def test_gpu_block_size_change_needs_the_natural_injection(case, hierarchies):
    """A hierarchy whose block size changes through any other P is refused at setup."""
    from fhhos4_gb300 import _native as N
    As, Ps, b, bss, cnu = hierarchies["ch"]
    P = Ps[0].copy()
    P.data[0] = 0.5
    with pytest.raises(N.FhgError) as e:
        _solver().fcg_mg(As, [P] + Ps[1:], bss, precision="fp64")
    assert e.value.code == N.FHG_ERR_UNSUPPORTED and "natural injection" in str(e.value)
