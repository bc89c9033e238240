"""Batched solve: many independent problems of uneven size (n, k and coefficient field differ)
solved by one graph launch with device-side WHILE loops must give, problem by problem, the
iteration counts, residuals and solutions of the individual solves (the launch sequence of each
problem is the same, residual replacement included: the loop body's IF node checks the true
residual once the recursive one meets the tolerance), and every solve is judged by its true
residual."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _specs():
    from fhhos4_gb300.batch import ProblemSpec
    # the last one has the deepest hierarchy of the batched workload (n = 256, k = 3: six levels, the
    # coarse ones in one cluster launch inside the graph's loop body)
    return [ProblemSpec(32, 1, 11), ProblemSpec(48, 3, 12), ProblemSpec(64, 2, 13), ProblemSpec(80, 1, 14),
            ProblemSpec(32, 2, 15), ProblemSpec(96, 3, 16), ProblemSpec(256, 3, 17)]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_matches_individual_solves(precision):
    from fhhos4_gb300 import batch as B
    probs, batch, _ = B.build(_specs(), precision=precision, autotune=False, keep_operator=True)
    try:
        # individual solves first (fhg_solve on the same contexts)
        ref = []
        for p in probs:
            rc, x, hist, info = p.ctx.solve(p.b, 200)
            assert rc == 0
            ref.append((x, info))
        for p in probs:
            p.upload_b()
        rc, infos, ms = batch.solve()
        assert rc == 0 and ms > 0
        for p, (x_ref, info_ref), info in zip(probs, ref, infos):
            assert info.status == 0
            x = p.x()
            r_true = np.linalg.norm(p.b - p.A0 @ x) / np.linalg.norm(p.b)
            # ||b - A x|| in FP64 has few significant digits at 1e-8 with a 1e6 coefficient contrast
            # (cancellation against |A||x|): compare to 1e-11 of ||b||
            assert info.true_relative_residual == pytest.approx(r_true, rel=1e-3, abs=1e-11)
            assert info.normalized_residual < 1e-8
            # the device loop replaces the residual as the individual FP32 solve does (true residual
            # checked once the recursive one meets the tolerance), so both run the same iterations
            assert info.iterations == info_ref.iterations
            assert info.normalized_residual == pytest.approx(info_ref.normalized_residual, rel=1e-12)
            assert np.linalg.norm(x - x_ref) <= 1e-12 * np.linalg.norm(x_ref)
            assert info.true_relative_residual == pytest.approx(info_ref.true_relative_residual, rel=1e-6, abs=1e-12)
            if precision == "fp32":
                assert info.true_relative_residual < 1e-8
            assert r_true < 1.5e-8
        # a second launch of the same graph gives the same answers
        rc2, infos2, _ = batch.solve()
        assert rc2 == 0
        assert [i.iterations for i in infos2] == [i.iterations for i in infos]
    finally:
        batch.close()
        for p in probs:
            p.close()


def test_batch_rebuilds_after_setup_and_stops_at_max_iterations():
    """A context set up again (here with max_iterations = 3) is picked up by the next batched solve,
    whose device-side loop then stops at 3 iterations."""
    from fhhos4_gb300 import _native as N
    from fhhos4_gb300 import batch as B
    probs, batch, _ = B.build(_specs()[:2], autotune=False)
    try:
        rc, infos, _ = batch.solve()
        assert rc == 0 and all(i.iterations > 3 for i in infos)
        p = probs[0]
        from fhhos4_gb300 import hho
        H = hho.Hierarchy(2, p.spec.n, p.spec.k, source="modes", coefficient="lognormal_patches", contrast=1e3,
                          checker_blocks=8, seed=p.spec.seed, max_coarse_rows=1000)
        p.ctx.set_level(0, p.bs, H.A(0))
        for l in range(H.levels - 1):
            p.ctx.set_prolongation(l, H.P(l))
        o = N.default_options()
        o.galerkin = 1
        o.max_iterations = 3
        p.ctx.setup(H.levels, o)
        H.close()
        p.upload_b()
        rc, infos, _ = batch.solve()
        assert rc == 0
        assert infos[0].iterations == 3 and infos[0].normalized_residual > 1e-8
        assert infos[1].iterations > 3
    finally:
        batch.close()
        for p in probs:
            p.close()


def test_batch_follows_cycle_and_precision_changes():
    """Changing the cycle or the V-cycle precision of a context in a batch makes the next batched
    solve capture the new launch sequence (the same iterations as the individual solve)."""
    from fhhos4_gb300 import batch as B
    probs, batch, _ = B.build(_specs()[:2], precision="fp32", autotune=False)
    try:
        rc, infos, _ = batch.solve()
        assert rc == 0
        for prec, nu in (("fp64", (1, 1)), ("fp32", (2, 2))):
            for p in probs:
                p.ctx.set_vcycle_precision(prec)
                p.ctx.set_cycle("bgs", "rbgs", nu[0], nu[1], 1)
            ref = [p.ctx.solve(p.b, 200)[3].iterations for p in probs]
            for p in probs:
                p.upload_b()
            rc, infos, _ = batch.solve()
            assert rc == 0
            assert [i.iterations for i in infos] == ref
    finally:
        batch.close()
        for p in probs:
            p.close()


def test_batch_rejects_unsupported_contexts():
    from fhhos4_gb300 import _native as N
    from fhhos4_gb300 import hho
    As, Ps, b, bs = hho.generate(2, 8, 1)
    ctx = N.Context(0)
    for l, A in enumerate(As):
        ctx.set_level(l, bs, A)
    for l, P in enumerate(Ps):
        ctx.set_prolongation(l, P)
    o = N.default_options()
    o.krylov = N.KRYLOV["cg"]
    ctx.setup(len(As), o)
    batch = N.Batch(0)
    with pytest.raises(N.FhgError) as ei:
        batch.add(ctx)
    assert ei.value.code == N.FHG_ERR_UNSUPPORTED
    batch.close()
    ctx.close()
