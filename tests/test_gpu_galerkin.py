"""Galerkin coarse operators (Multigrid::UseGalerkinOperator, "-g 1"; Level.h:133-137):
A_{l+1} = P_l^T A_l P_l formed at setup. Checked against the triple product formed by scipy and
against the oracle's solve on that hierarchy in the GPU's colour order; the high-contrast case is
the one the rediscretised hierarchy cannot solve."""
import numpy as np
import pytest

import oracle as O
from test_oracle import hist_close

pytestmark = pytest.mark.gpu


def _hier(n, k, coefficient="identity", contrast=1.0):
    from fhhos4_gb300 import hho
    H = hho.Hierarchy(3, n, k, coefficient=coefficient, contrast=contrast, checker_blocks=4,
                      source="one" if coefficient != "identity" else "sine", max_coarse_rows=1000)
    As = [H.A(l) for l in range(H.levels)]
    Ps = [H.P(l) for l in range(H.levels - 1)]
    b, bs = H.b(), H.block_size
    H.close()
    return As, Ps, b, bs


def _galerkin(As, Ps):
    Ag = [As[0].tocsr()]
    for P in Ps:
        Ag.append((P.T @ Ag[-1] @ P).tocsr())
    return Ag


def _context(As, Ps, bs, precision="fp64", only_fine=True):
    from fhhos4_gb300 import _native as N
    ctx = N.Context(0)
    ctx.set_level(0, bs, As[0])
    if not only_fine:
        for l in range(1, len(As)):
            ctx.set_level(l, bs, As[l])
    for l, P in enumerate(Ps):
        ctx.set_prolongation(l, P)
    o = N.default_options()
    o.galerkin = 1
    o.vcycle_precision = N.PRECISION[precision]
    ctx.setup(len(As), o)
    return ctx, o


def test_galerkin_operators_are_the_triple_product():
    from fhhos4_gb300 import _native as N
    As, Ps, b, bs = _hier(8, 2)
    Ag = _galerkin(As, Ps)
    ctx, _ = _context(As, Ps, bs, only_fine=True)
    rng = np.random.default_rng(0)
    for l in range(1, len(As)):
        x = rng.standard_normal(Ag[l].shape[0])
        y = ctx.apply(l, N.OP_SPMV, x, None, Ag[l].shape[0])
        ref = Ag[l] @ x
        assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-13
    ctx.close()


def test_galerkin_replaces_given_coarse_operators():
    from fhhos4_gb300 import _native as N
    As, Ps, b, bs = _hier(8, 2)
    Ag = _galerkin(As, Ps)
    ctx, o = _context(As, Ps, bs, only_fine=False)   # rediscretised operators given, then replaced
    x = np.random.default_rng(1).standard_normal(Ag[1].shape[0])
    y = ctx.apply(1, N.OP_SPMV, x, None, Ag[1].shape[0])
    assert np.linalg.norm(y - Ag[1] @ x) / np.linalg.norm(Ag[1] @ x) < 1e-13
    # a later setup without Galerkin refuses the replaced operators until they are set again
    o.galerkin = 0
    with pytest.raises(N.FhgError):
        ctx.setup(len(As), o)
    for l in range(1, len(As)):
        ctx.set_level(l, bs, As[l])
    ctx.setup(len(As), o)
    ctx.close()


def test_galerkin_solve_matches_oracle_in_colour_order():
    from fhhos4_gb300 import solver as S
    As, Ps, b, bs = _hier(8, 2)
    Ag = _galerkin(As, Ps)
    perms, _ = O.colour_perms(Ag, bs)
    Ac, Pc, bc = O.permute_hierarchy(Ag, Ps, b, bs, perms)
    x_o, hist_o, its_o, st = O.fcgmg_solve(Ac, Pc, bc, bs)
    assert st == 0
    fcg = S.fcg_mg(As, Ps, bs, galerkin=True)
    x = fcg.Solve(b)
    assert fcg.IterationCount == its_o
    assert hist_close(fcg.History, hist_o[: its_o + 1])
    ctx = fcg.Context()
    for l in range(len(As) - 1):
        assert np.array_equal(ctx.permutation(l, Ag[l].shape[0] // bs), perms[l])
    sp_ = (np.asarray(perms[0])[:, None] * bs + np.arange(bs)).ravel()
    assert np.linalg.norm(x[sp_] - x_o) / np.linalg.norm(x_o) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_high_contrast_checkerboard_converges_with_galerkin(precision):
    """Checkerboard 1 / 1e6 on 4x4x4 blocks, k = 2: the rediscretised hierarchy does not converge
    (oracle), the Galerkin one does, in both V-cycle precisions; the FP64 true residual judges it."""
    from fhhos4_gb300 import solver as S
    As, Ps, b, bs = _hier(8, 2, coefficient="checkerboard", contrast=1e6)
    _, hist_r, its_r, _ = O.fcgmg_solve(As, Ps, b, bs, maxit=60)
    assert its_r == 60 and hist_r[-1] > 1e-3       # rediscretised: no convergence
    Ag = _galerkin(As, Ps)
    perms, _ = O.colour_perms(Ag, bs)
    Ac, Pc, bc = O.permute_hierarchy(Ag, Ps, b, bs, perms)
    _, hist_o, its_o, _ = O.fcgmg_solve(Ac, Pc, bc, bs, maxit=300)
    fcg = S.fcg_mg(As, Ps, bs, galerkin=True, precision=precision, maxit=300)
    x = fcg.Solve(b)
    assert fcg.History[-1] < 1e-8
    r = np.linalg.norm(b - As[0] @ x) / np.linalg.norm(b)
    if precision == "fp64":
        assert fcg.IterationCount == its_o
        assert r < 1.5e-8
    else:
        # FP32 V-cycle: residual replacement makes the FP64 true residual meet the tolerance
        assert fcg.IterationCount <= its_o + 40
        assert r < 1e-8 * (1 + 1e-6)


@pytest.mark.parametrize("precision", ["fp64", "df", "fp32"])
def test_high_contrast_true_residual_meets_tolerance_with_replacement(precision):
    """Checkerboard 1 / 1e6, k = 2: a plain FP64 evaluation of b - A x errs by about
    u sum |a_ij x_j|, 2e7 times ||b|| here. With residual replacement on (and the true residual that
    misses the tolerance evaluated again in compensated arithmetic), every precision returns an x
    whose true residual, evaluated on the host in extended precision, meets 1e-8."""
    from fhhos4_gb300 import solver as S
    As, Ps, b, bs = _hier(8, 2, coefficient="checkerboard", contrast=1e6)
    fcg = S.fcg_mg(As, Ps, bs, galerkin=True, precision=precision, maxit=300, replace_residual=True)
    x = fcg.Solve(b)
    A = As[0].tocsr()
    Al = A.astype(np.longdouble)
    r = np.asarray(b, dtype=np.longdouble) - Al @ np.asarray(x, dtype=np.longdouble)
    true_ext = float(np.sqrt(np.sum(r * r)) / np.linalg.norm(b))
    assert true_ext < 1e-8, true_ext
    assert fcg.TrueRelativeResidual < 1e-8
    assert abs(fcg.TrueRelativeResidual - true_ext) <= 0.05 * true_ext + 1e-12
