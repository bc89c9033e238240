"""Full-size parity: the hierarchy generated on the host at 16^3, 32^3 and the benchmark's 64^3
(9,363,456 unknowns), solved on the GPU, against the reference's own residual histories for the
same problem in the same colour order (tests/golden/tet3d_n*_k1.npz, generated by the
reference). Size-independent properties checked alongside: exact iteration count, history
within 1e-10 relative per iteration, FP64 true residual below the tolerance, FP32 V-cycle
reaching the same FP64 tolerance, the pair (FP64-class) V-cycle at the reference's bar,
bitwise-reproducible repeated solves.
"""
import numpy as np
import pytest

from _golden import Case, available
from test_oracle import hist_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=available(["tet3d_n16_k1", "tet3d_n32_k1", "tet3d_n64_k1"]))
def problem(request):
    from fhhos4_gb300 import hho
    c = Case(request.param)
    As, Ps, b, bs = hho.generate(3, c.n, 1)
    return c, As, Ps, b, bs


def test_generated_hierarchy_solve_matches_reference_history(problem):
    from fhhos4_gb300 import _native as N
    from fhhos4_gb300 import solver as S
    c, As, Ps, b, bs = problem
    assert [A.shape[0] for A in As] == list(c["level_rows"])
    fcg = S.fcg_mg(As, Ps, bs, precision="fp32", extra=("df",))   # FP64, FP32 and pair operators
    ctx = fcg.Context()
    ctx.set_vcycle_precision("fp64")
    x = fcg.Solve(b)
    ref = np.asarray(c["hist_colour"])
    assert fcg.IterationCount == len(ref) - 1
    assert hist_close(fcg.History, ref), np.max(np.abs(fcg.History - ref) / ref)
    r = ctx.apply(0, N.OP_RESIDUAL, x, b, len(b))
    assert np.linalg.norm(r) / np.linalg.norm(b) < 1e-8 * 1.01
    x2 = fcg.Solve(b)
    assert np.array_equal(x, x2)
    # FP32 V-cycle inside FP64 FCG reaches the same FP64 tolerance
    ctx.set_vcycle_precision("fp32")
    x32 = fcg.Solve(b)
    assert fcg.History[-1] < 1e-8
    assert fcg.IterationCount <= len(ref) + 2
    r32 = ctx.apply(0, N.OP_RESIDUAL, x32, b, len(b))
    assert np.linalg.norm(r32) / np.linalg.norm(b) < 2e-8
    assert np.linalg.norm(x32 - x) / np.linalg.norm(x) < 1e-6
    # the pair V-cycle (FP64-class arithmetic on the FP32 pipe) at the reference's bar
    ctx.set_vcycle_precision("df")
    xdf = fcg.Solve(b)
    assert fcg.IterationCount == len(ref) - 1
    assert hist_close(fcg.History, ref), np.max(np.abs(fcg.History - ref) / ref)
    rdf = ctx.apply(0, N.OP_RESIDUAL, xdf, b, len(b))
    assert np.linalg.norm(rdf) / np.linalg.norm(b) < 1e-8 * 1.01
    assert np.linalg.norm(xdf - x) / np.linalg.norm(x) < 1e-10
