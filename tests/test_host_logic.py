"""Host-side logic of the Python mirror that needs no GPU: option mapping, argument checks,
unsupported configurations failing loudly."""
import numpy as np
import pytest
import scipy.sparse as sp

from fhhos4_gb300 import _native as N
from fhhos4_gb300 import solver as S


def test_as_eigen_csr_is_canonical():
    A = sp.coo_matrix((np.array([1.0, 2.0, 3.0]), (np.array([1, 0, 1]), np.array([0, 1, 0]))), shape=(2, 2))
    C = S.as_eigen_csr(A)
    assert C.indptr.dtype == np.int32 and C.indices.dtype == np.int32
    assert C[1, 0] == 4.0 and C.nnz == 2


def test_reference_defaults_are_mirrored():
    fcg = S.FlexibleConjugateGradient()
    assert fcg.Truncation == 1 and not fcg.Restart
    mg = S.Multigrid()
    assert (mg.PreSmootherCode, mg.PostSmootherCode) == ("bgs", "rbgs")
    assert (mg.PreSmoothingIterations, mg.PostSmoothingIterations) == (1, 1)
    assert mg.Cycle == "V" and mg.MatrixMaxSizeForCoarsestLevel == 1000
    assert fcg.MaxIterations == 200


def test_unsupported_configurations_fail_loudly():
    with pytest.raises(NotImplementedError):
        S.FlexibleConjugateGradient(truncation=2)
    mg = S.Multigrid()
    mg.Cycle = "K"
    mg._check_supported()           # V, W and K run on the GPU
    mg.Cycle = "F"                  # no such cycle in the reference
    with pytest.raises(NotImplementedError):
        mg._check_supported()
    mg.Cycle = "V"
    for code in ("hbgs", "hrbgs", "bsor", "rbsor", "sbsor", "absor", "rabsor"):
        mg.PreSmootherCode = code       # aliases of the GPU Gauss-Seidel codes
        mg._check_supported()
    mg.PreSmootherCode = "gs"           # point (scalar) Gauss-Seidel: block size 1 only
    with pytest.raises(NotImplementedError):
        mg._check_supported()
    fcg = S.FlexibleConjugateGradient()
    with pytest.raises(NotImplementedError):
        fcg.Setup(sp.identity(4, format="csr"))   # no multigrid preconditioner


def test_hierarchy_shape_checks():
    mg = S.Multigrid()
    with pytest.raises(ValueError):
        mg.SetHierarchy([sp.identity(6)], [sp.identity(6)])


def test_option_codes_match_header():
    assert N.SMOOTHERS == {"bgs": 0, "rbgs": 1, "bj": 2, "bj23": 3, "sbgs": 4, "abgs": 5, "rabgs": 6}
    assert N.KRYLOV == {"fcg": 0, "cg": 1}
    assert N.PRECISION == {"fp64": 0, "fp32": 1, "df": 2}


def test_batched_workload_is_seeded_and_in_range():
    """The batched workload: 2D problems with n a multiple of 16 in [32, 256], k in {1, 2, 3}, the
    same draw for the same seed."""
    from fhhos4_gb300 import batch as B
    a, b = B.batched_specs(64), B.batched_specs(64)
    assert [(s.n, s.k, s.seed) for s in a] == [(s.n, s.k, s.seed) for s in b]
    assert all(32 <= s.n <= 256 and s.n % 16 == 0 and s.k in (1, 2, 3) for s in a)
    assert len({s.seed for s in a}) == len(a)


def test_bench_workloads_are_named_for_what_they_are():
    """Every extra workload of the bench line carries its mesh, degree and coefficient in its key and
    lists the methods it compares; the workload record of the line names sizes, not an index."""
    import argparse
    import bench
    for key, spec in bench.EXTRA_CONFIGS.items():
        assert key.startswith(f"tet{spec['n']}_k{spec['k']}_"), key
        assert spec["methods"] and all(len(m) == 7 for m in spec["methods"].values())
    args = argparse.Namespace(dim=3, n=64, k=1, coefficient="identity", contrast=1.0, source="sine",
                              max_coarse_rows=1000, galerkin=False, checker_blocks=4, seed=0)
    w = bench.workload_config(args, 9363456, 6)
    assert "64^3" in w["workload"] and w["unknowns"] == 9363456
