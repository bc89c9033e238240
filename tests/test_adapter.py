"""The C++ adapter (include/fhg_reference_adapter.hpp) compiled against the reference's headers:
ProgramArguments -> fhg_options as the reference's SolverFactory reads them (SolverFactory.h:125-200,
236-310; SmootherFactory.h:37-100). CPU only: `adapter_check --map` makes no GPU call. Skipped
where the reference checkout or libfhg.so is absent."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = os.environ.get("FHHOS4_REFERENCE", "/root/reference")
LIB = os.path.join(ROOT, "fhhos4_gb300", "_build", "libfhg.so")


def _mapped():
    if not os.path.isdir(os.path.join(REFERENCE, "src", "Solver")):
        pytest.skip("reference checkout not present")
    if not os.path.exists(LIB):
        pytest.skip("libfhg.so not built")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "adapter", f"REF_ROOT={REFERENCE}"],
                   check=True, timeout=600)
    out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "adapter_check"), "--map"], check=True,
                         capture_output=True, text=True, timeout=60).stdout
    rows = {}
    for line in out.splitlines():
        name, *kv = line.split()
        rows[name] = {k: v for k, v in (x.split("=") for x in kv)}
    return rows


def test_adapter_argument_mapping():
    m = _mapped()
    # fcgmg defaults: V(1,1), bgs / rbgs, omega 1, tolerance 1e-8, 200 iterations (ProgramArguments.h:60-95)
    assert m["default"] == dict(krylov="0", pre="0", post="1", npre="1", npost="1", omega="1", w_loops="1",
                                galerkin="0", tol="1e-08", maxit="200", cpre="-1", cpost="-1")
    # "<symmetric smoother>" after abgs with an odd step count is "rabgs" (SolverFactory.h:270-280)
    assert (m["abgs3_symmetric"]["pre"], m["abgs3_symmetric"]["post"]) == ("5", "6")
    # hbgs -> hrbgs, both the multicolour forward / backward sweeps
    assert (m["hbgs_symmetric"]["pre"], m["hbgs_symmetric"]["post"]) == ("0", "1")
    # cg + mg preconditioner, W-cycle, Galerkin, block SOR aliases with omega 1.2
    w = m["cg_w_sor"]
    assert (w["krylov"], w["w_loops"], w["galerkin"], w["pre"], w["post"], w["omega"]) == ("1", "2", "1", "0", "1", "1.2")
    assert (w["tol"], w["maxit"]) == ("1e-10", "50")
    # cgmg, K-cycle, bj23 symmetric post-smoother is bj23 itself
    k = m["cgmg_k_bj23"]
    assert (k["krylov"], k["w_loops"], k["pre"], k["post"]) == ("1", "-1", "3", "3")
    # the p-multigrid preconditioner (SolverFactory.h:201-211): direct coarse solve by default; with
    # "-cs mg" one h-multigrid cycle, V(0, 3) in 2D, below the lowest degree (SolverFactory.h:299-308)
    assert m["fcgp_mg"] == dict(m["default"])
    c = m["cg_p_mg_cs_mg"]
    assert (c["krylov"], c["cpre"], c["cpost"], c["npre"], c["npost"]) == ("1", "0", "3", "1", "1")


@pytest.mark.parametrize("what", ["solver", "smoother", "coarse", "variable", "coarse_mg", "p_mg_w"])
def test_adapter_rejects_unsupported(what):
    _mapped()
    p = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "adapter_check"), "--reject", what],
                       capture_output=True, text=True, timeout=60)
    assert p.returncode != 0 and "accepted" not in p.stdout
    assert "GPU solver" in p.stdout + p.stderr


def _levels(*argv):
    _mapped()
    p = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "adapter_check"), "--levels", *map(str, argv)],
                       check=True, capture_output=True, text=True, timeout=300)
    rows = []
    for line in p.stderr.splitlines():
        if line.startswith("level"):
            rows.append({k: int(v) for k, v in (x.split("=") for x in line.split()[1:])})
    return rows


@pytest.mark.parametrize("cs", ["ch", "mg"])
def test_adapter_builds_the_p_multigrid_hierarchy(cs):
    """The adapter's host side (no device call): the reference's P_MultigridForHHO levels (and, for
    "-cs mg", its coarse multigrid's levels below the lowest degree) with their block sizes and
    prolongations, the hierarchy hho.generate_p builds for the same problem."""
    from fhhos4_gb300 import hho
    got = _levels(2, 16, 3, "fcgp_mg", cs)
    As, Ps, b, bss, _ = hho.generate_p(2, 16, 3, cs)
    assert [r["rows"] for r in got] == [A.shape[0] for A in As]
    assert [r["bs"] for r in got] == bss
    assert [(r["p_rows"], r["p_cols"]) for r in got] == [P.shape for P in Ps] + [(0, 0)]


def test_adapter_builds_the_h_multigrid_hierarchy():
    from fhhos4_gb300 import hho
    got = _levels(2, 32, 1, "fcgmg", "ch")
    H = hho.Hierarchy(2, 32, 1)
    try:
        assert [r["rows"] for r in got] == [H.A_rows(l) for l in range(H.levels)]
        assert all(r["bs"] == H.block_size for r in got)
    finally:
        H.close()

