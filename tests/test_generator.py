"""The host hierarchy producer (csrc/hho_gen.cpp) against the reference's own hierarchies.

A_l and P_l on every level must equal the reference's to rounding (1e-13 relative to the
largest entry). b differs only by the reference's source-term quadrature (a degree-8 rule on
each tetrahedron; this generator integrates to machine precision), an error that decays like
h^9: bounded per case below. On triangles both rules are exact to rounding. CPU only.
"""
import numpy as np
import pytest

import oracle as O
from _golden import FULL_CASES, Case, available
from test_oracle import hist_close

from fhhos4_gb300 import hho

B_TOL = {(2, None): 1e-13, (3, 4): 1e-7, (3, 8): 1e-10}


@pytest.fixture(scope="module", params=available(FULL_CASES))
def case(request):
    return Case(request.param)


@pytest.fixture(scope="module")
def generated(case):
    return hho.generate(case.dim, case.n, case.k)


def test_same_hierarchy_shape(case, generated):
    As, Ps, b, bs = generated
    assert bs == case.bs
    assert len(As) == case.levels
    assert [A.shape[0] for A in As] == list(case["level_rows"])


def test_operators_match_reference(case, generated):
    As, Ps, b, bs = generated
    for l in range(case.levels):
        ref = case.As[l]
        assert abs(As[l] - ref).max() <= 1e-13 * abs(ref).max(), l
    for l in range(case.levels - 1):
        ref = case.Ps[l]
        assert Ps[l].shape == ref.shape
        assert abs(Ps[l] - ref).max() <= 1e-13 * abs(ref).max(), l


def test_rhs_matches_reference(case, generated):
    As, Ps, b, bs = generated
    tol = B_TOL[(2, None)] if case.dim == 2 else B_TOL[(3, case.n)]
    assert np.linalg.norm(b - case.b) <= tol * np.linalg.norm(case.b)


def test_block_pattern_is_the_reference_one(case, generated):
    # Integer structure: block-level sparsity of every A_l (what colouring and BSR depend on).
    As, Ps, b, bs = generated
    for l in range(case.levels):
        def blocks(A):
            A = A.tocoo()
            return set(zip((A.row // bs).tolist(), (A.col // bs).tolist()))
        assert blocks(As[l]) == blocks(case.As[l])


@pytest.mark.parametrize("name", available(["tet3d_n16_k1"]))
def test_generated_16cube_reproduces_reference_history(name):
    c = Case(name)
    As, Ps, b, bs = hho.generate(3, 16, 1)
    assert [A.shape[0] for A in As] == list(c["level_rows"])
    perms, ncol = O.colour_perms(As, bs)
    Ac, Pc, bc = O.permute_hierarchy(As, Ps, b, bs, perms)
    x, hist, it, rc = O.fcgmg_solve(Ac, Pc, bc, bs)
    ref = np.asarray(c["hist_colour"])
    assert rc == 0 and it == len(ref) - 1
    assert hist_close(hist, ref)


def test_l2_error_post_processing_matches_reference(case, generated):
    # Cell recovery + k+1 reconstruction + relative L2 error against the exact solution, applied to
    # the reference's own solution: equal to the reference's L2Error up to the two quadratures
    # (exact to rounding on triangles; degree-8 rule on tetrahedra, larger gap on the coarsest mesh).
    from fhhos4_gb300 import hho
    ref = float(case["l2_error"])
    H = hho.Hierarchy(case.dim, case.n, case.k)
    e = H.l2_error(case["x_natural"])
    H.close()
    tol = 1e-8 if case.dim == 2 else (1e-3 if case.n <= 4 else 1e-5)
    assert abs(e - ref) <= tol * ref
