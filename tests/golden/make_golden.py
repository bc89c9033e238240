"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference harness (oracle/_ref/ref_driver, compiled from the reference
checkout by ``make -C oracle ref``) and stores, per case, in a compressed .npz:

* the whole multigrid hierarchy the reference builds (A_l, P_l as CSR) and b;
* the reference FCG(1)+V(1,1) residual history and solution in its natural
  block-Gauss-Seidel order (``hist_natural``, ``x_natural``);
* the colour permutation of every level computed by the oracle's greedy
  colouring, and the reference's own classes re-run on the colour-permuted
  hierarchy (``hist_colour``, ``x_colour`` in the permuted numbering), for
  block GS (bgs/rbgs), block Jacobi (bj23), PCG (``cg``), the W-cycle (``w``), symmetric block
  GS (``sbgs``) and alternating block GS (``abgs``/``rabgs``); ``--add-k-cycle`` adds the K-cycle
  (``hist_k``, ``x_k``) to existing full cases.

Only ``hist_*`` summaries are kept for the large cases (``--histories-only``).

``--add-sor`` adds the reference's block SOR (bsor/rbsor and sbsor, omega 1.2) to full cases.

``--p-multigrid`` writes the p-multigrid cases (``p_*.npz``): the reference's FCG with its
p-multigrid preconditioner ("-s fcg -p p_mg", P_MultigridForHHO) with the coarse solvers "ch" and
"mg" (``hist_ch``/``x_ch``, ``hist_mg``/``x_mg``), the block size of every level, and per level
A_l v_l for a seeded v_l (``Av{l}``) with A_l's shape and entry count instead of A_l itself.
The 2D case also holds the strategy Minus1 with "ch" (degrees 3, 2, 1: ``hist_ch_minus1``,
``x_ch_minus1``, ``block_sizes_ch_minus1``).

Usage:  python tests/golden/make_golden.py [case ...] [--histories-only | --add-k-cycle | --add-sor]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np
import scipy.sparse as sp

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402

GOLDEN = os.path.dirname(os.path.abspath(__file__))

# name -> (dim, n, k)
CASES = {
    "tri2d_n8_k1": (2, 8, 1),
    "tri2d_n32_k1": (2, 32, 1),      # 2D Poisson, 2048 triangles, k=1
    "tri2d_n50_k1": (2, 50, 1),      # odd coarse n (25): hierarchy stops early, large coarsest
    "tri2d_n16_k2": (2, 16, 2),      # block size 3
    "tet3d_n4_k1": (3, 4, 1),
    "tet3d_n8_k1": (3, 8, 1),
    "tet3d_n4_k2": (3, 4, 2),        # block size 6
}
LARGE = {
    "tet3d_n16_k1": (3, 16, 1),
    "tet3d_n32_k1": (3, 32, 1),
    "tet3d_n64_k1": (3, 64, 1),
}


def load_csr(prefix):
    sh = np.fromfile(prefix + "_shape.i32", dtype=np.int32)
    rp = np.fromfile(prefix + "_rowptr.i32", dtype=np.int32)
    ci = np.fromfile(prefix + "_colidx.i32", dtype=np.int32)
    va = np.fromfile(prefix + "_vals.f64")
    return sp.csr_matrix((va, ci, rp), shape=(int(sh[0]), int(sh[1])))


def dump_csr(prefix, A):
    A = O.as_csr(A)
    np.asarray(A.shape, dtype=np.int32).tofile(prefix + "_shape.i32")
    A.indptr.astype(np.int32).tofile(prefix + "_rowptr.i32")
    A.indices.astype(np.int32).tofile(prefix + "_colidx.i32")
    A.data.astype(np.float64).tofile(prefix + "_vals.f64")


def ref_gen(dim, n, k, out):
    subprocess.run([O.REF_DRIVER, "gen", str(dim), str(n), str(k), out], check=True)
    meta = json.load(open(os.path.join(out, "meta.json")))
    L = meta["levels"]
    As = [load_csr(f"{out}/L{l}_A") for l in range(L)]
    Ps = [load_csr(f"{out}/L{l}_P") for l in range(L - 1)]
    b = np.fromfile(f"{out}/b.f64")
    return meta, As, Ps, b, np.fromfile(f"{out}/history.f64"), np.fromfile(f"{out}/x.f64")


def ref_solve(As, Ps, b, bs, work, smoothers="bgs,rbgs", krylov="fcg", cycle="V", omega=1.0):
    os.makedirs(work, exist_ok=True)
    np.asarray([len(As), bs], dtype=np.int32).tofile(f"{work}/levels.i32")
    for l, A in enumerate(As):
        dump_csr(f"{work}/L{l}_A", A)
    for l, P in enumerate(Ps):
        dump_csr(f"{work}/L{l}_P", P)
    np.asarray(b, dtype=np.float64).tofile(f"{work}/b.f64")
    subprocess.run([O.REF_DRIVER, "solve", work, "--smoothers", smoothers, "--krylov", krylov, "--cycle", cycle,
                    "--omega", repr(float(omega))], check=True)
    return np.fromfile(f"{work}/out_history.f64"), np.fromfile(f"{work}/out_x.f64")


def make_case(name, dim, n, k, histories_only=False):
    with tempfile.TemporaryDirectory() as tmp:
        gen = os.path.join(tmp, "gen")
        os.makedirs(gen)
        meta, As, Ps, b, hist_nat, x_nat = ref_gen(dim, n, k, gen)
        bs = meta["block_size"]
        perms, ncol = O.colour_perms(As, bs)
        Ac, Pc, bc = O.permute_hierarchy(As, Ps, b, bs, perms)
        hist_col, x_col = ref_solve(Ac, Pc, bc, bs, os.path.join(tmp, "col"))
        hist_bj, x_bj = ref_solve(Ac, Pc, bc, bs, os.path.join(tmp, "bj"), smoothers="bj23,bj23")
        hist_cg, x_cg = ref_solve(Ac, Pc, bc, bs, os.path.join(tmp, "cg"), krylov="cg")
        hist_w, x_w = ref_solve(Ac, Pc, bc, bs, os.path.join(tmp, "w"), cycle="W")
        hist_sbgs, x_sbgs = ref_solve(Ac, Pc, bc, bs, os.path.join(tmp, "sbgs"), smoothers="sbgs,sbgs")
        hist_abgs, x_abgs = ref_solve(Ac, Pc, bc, bs, os.path.join(tmp, "abgs"), smoothers="abgs,rabgs")
        out = dict(
            dim=dim, n=n, k=k, block_size=bs, levels=len(As),
            hist_natural=hist_nat, hist_colour=hist_col, hist_bj23=hist_bj, hist_cg=hist_cg,
            hist_w=hist_w, hist_sbgs=hist_sbgs, hist_abgs=hist_abgs,
            ncolours=np.asarray(ncol, dtype=np.int32),
            level_rows=np.asarray([A.shape[0] for A in As], dtype=np.int64),
            level_nnz=np.asarray([A.nnz for A in As], dtype=np.int64),
            p_nnz=np.asarray([P.nnz for P in Ps], dtype=np.int64),
            b_norm=np.linalg.norm(b), x_natural_norm=np.linalg.norm(x_nat),
            setup_s=meta.get("setup_s", 0.0), solve_s=meta.get("solve_s", 0.0),
            l2_error=meta.get("l2_error", float("nan")),
        )
        if not histories_only:
            out.update(b=b, x_natural=x_nat, x_colour=x_col, x_bj23=x_bj, x_cg=x_cg, x_w=x_w, x_sbgs=x_sbgs,
                       x_abgs=x_abgs)
            for l, A in enumerate(As):
                A = O.as_csr(A)
                out[f"A{l}_indptr"], out[f"A{l}_indices"], out[f"A{l}_data"] = A.indptr, A.indices, A.data
                out[f"perm{l}"] = perms[l]
            for l, P in enumerate(Ps):
                P = O.as_csr(P)
                out[f"P{l}_indptr"], out[f"P{l}_indices"], out[f"P{l}_data"] = P.indptr, P.indices, P.data
                out[f"P{l}_shape"] = np.asarray(P.shape, dtype=np.int64)
        path = os.path.join(GOLDEN, name + ".npz")
        np.savez_compressed(path, **out)
        print(f"{name}: levels={len(As)} N={As[0].shape[0]} nnz={As[0].nnz} iters nat/col/bj/cg="
              f"{len(hist_nat)-1}/{len(hist_col)-1}/{len(hist_bj)-1}/{len(hist_cg)-1} "
              f"size={os.path.getsize(path)/1e6:.2f} MB", flush=True)


# Block SOR fixtures: the reference's BlockSOR (BlockSOR.h:99-227) through the bsor/rbsor and
# sbsor codes with relaxation parameter SOR_OMEGA, on the colour-permuted hierarchy.
SOR_OMEGA = 1.2


def _load_full(name):
    path = os.path.join(GOLDEN, name + ".npz")
    with np.load(path) as z:
        data = {k: z[k] for k in z.files}
    nl = int(data["levels"])
    bs = int(data["block_size"])
    As = [sp.csr_matrix((data[f"A{l}_data"], data[f"A{l}_indices"], data[f"A{l}_indptr"])) for l in range(nl)]
    Ps = [sp.csr_matrix((data[f"P{l}_data"], data[f"P{l}_indices"], data[f"P{l}_indptr"]),
                        shape=tuple(data[f"P{l}_shape"])) for l in range(nl - 1)]
    perms = [data[f"perm{l}"] for l in range(nl)]
    Ac, Pc, bc = O.permute_hierarchy(As, Ps, data["b"], bs, perms)
    return path, data, bs, Ac, Pc, bc


def add_sor(name):
    """Add block SOR (bsor/rbsor and sbsor, omega = SOR_OMEGA) of the reference on the stored
    colour-permuted hierarchy of a full case: hist_sor, x_sor, hist_ssor, x_ssor."""
    path, data, bs, Ac, Pc, bc = _load_full(name)
    with tempfile.TemporaryDirectory() as tmp:
        hist_sor, x_sor = ref_solve(Ac, Pc, bc, bs, os.path.join(tmp, "sor"), smoothers="bsor,rbsor", omega=SOR_OMEGA)
        hist_ssor, x_ssor = ref_solve(Ac, Pc, bc, bs, os.path.join(tmp, "ssor"), smoothers="sbsor,sbsor",
                                      omega=SOR_OMEGA)
    data.update(hist_sor=hist_sor, x_sor=x_sor, hist_ssor=hist_ssor, x_ssor=x_ssor, sor_omega=SOR_OMEGA)
    np.savez_compressed(path, **data)
    print(f"{name}: block SOR iterations {len(hist_sor) - 1}, symmetric {len(hist_ssor) - 1}", flush=True)


def add_k_cycle(name):
    """Add the reference's K-cycle (FCG(1) + K,1,1, bgs/rbgs; Multigrid.h:523-537,611-656) on the
    stored colour-permuted hierarchy of a full case: hist_k, x_k."""
    path = os.path.join(GOLDEN, name + ".npz")
    with np.load(path) as z:
        data = {k: z[k] for k in z.files}
    nl = int(data["levels"])
    bs = int(data["block_size"])
    As = [sp.csr_matrix((data[f"A{l}_data"], data[f"A{l}_indices"], data[f"A{l}_indptr"])) for l in range(nl)]
    Ps = [sp.csr_matrix((data[f"P{l}_data"], data[f"P{l}_indices"], data[f"P{l}_indptr"]),
                        shape=tuple(data[f"P{l}_shape"])) for l in range(nl - 1)]
    perms = [data[f"perm{l}"] for l in range(nl)]
    Ac, Pc, bc = O.permute_hierarchy(As, Ps, data["b"], bs, perms)
    with tempfile.TemporaryDirectory() as tmp:
        hist_k, x_k = ref_solve(Ac, Pc, bc, bs, os.path.join(tmp, "k"), cycle="K")
    data.update(hist_k=hist_k, x_k=x_k)
    np.savez_compressed(path, **data)
    print(f"{name}: K-cycle iterations {len(hist_k) - 1}", flush=True)


# name -> (dim, n, k): face degree k lowered to 1 on the same mesh (P_CS Minus2, CoarsePolyDegree 1)
P_CASES = {
    "p_tri2d_n16_k3": (2, 16, 3),    # block sizes 4 -> 2
    "p_tet3d_n4_k2": (3, 4, 2),      # block sizes 6 -> 3
}


def probe_vector(l, n):
    """The seeded vector the fixtures multiply level l's operator with."""
    return np.random.default_rng(1000 + l).standard_normal(n)


def make_p_case(name, dim, n, k):
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for cs in ("ch", "mg"):
            d = os.path.join(tmp, cs)
            os.makedirs(d)
            subprocess.run([O.REF_DRIVER, "genp", str(dim), str(n), str(k), d, "--coarse-solver", cs], check=True)
            meta = json.load(open(os.path.join(d, "meta.json")))
            out[f"hist_{cs}"] = np.fromfile(f"{d}/history.f64")
            out[f"x_{cs}"] = np.fromfile(f"{d}/x.f64")
            out[f"levels_{cs}"] = meta["levels"]
            if cs == "mg":
                L = meta["levels"]
                out["block_sizes"] = np.fromfile(f"{d}/block_sizes.i32", dtype=np.int32)
                out["p_levels"] = meta["p_levels"]
                out["b"] = np.fromfile(f"{d}/b.f64")
                for l in range(L):
                    A = load_csr(f"{d}/L{l}_A")
                    out[f"A{l}_shape"] = np.asarray(A.shape, dtype=np.int64)
                    out[f"A{l}_nnz"] = A.nnz
                    out[f"Av{l}"] = A @ probe_vector(l, A.shape[0])
                for l in range(L - 1):
                    P = load_csr(f"{d}/L{l}_P")
                    out[f"P{l}_shape"] = np.asarray(P.shape, dtype=np.int64)
                    out[f"P{l}_nnz"] = P.nnz
                    out[f"Pv{l}"] = P @ probe_vector(100 + l, P.shape[1])
        if dim == 2:
            d = os.path.join(tmp, "minus1")
            os.makedirs(d)
            subprocess.run([O.REF_DRIVER, "genp", str(dim), str(n), str(k), d, "--coarse-solver", "ch",
                            "--p-cs", "minus1"], check=True)
            out["hist_ch_minus1"] = np.fromfile(f"{d}/history.f64")
            out["x_ch_minus1"] = np.fromfile(f"{d}/x.f64")
            out["block_sizes_ch_minus1"] = np.fromfile(f"{d}/block_sizes.i32", dtype=np.int32)
    out.update(dim=dim, n=n, k=k)
    path = os.path.join(GOLDEN, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{name}: block sizes {[int(v) for v in out['block_sizes']]}, iterations ch/mg {len(out['hist_ch']) - 1}/"
          f"{len(out['hist_mg']) - 1}, size={os.path.getsize(path) / 1e6:.2f} MB", flush=True)


def build_ref_driver():
    """The reference harness, compiled from the read-only reference checkout (FHHOS4_REFERENCE)."""
    ref = os.environ.get("FHHOS4_REFERENCE", "/root/reference")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF_ROOT={ref}"], check=True)


def main(argv):
    histories_only = "--histories-only" in argv
    if "--p-multigrid" in argv:
        build_ref_driver()
        for name in [a for a in argv if not a.startswith("--")] or list(P_CASES):
            make_p_case(name, *P_CASES[name])
        return
    for flag, fn in (("--add-k-cycle", add_k_cycle), ("--add-sor", add_sor)):
        if flag in argv:
            build_ref_driver()
            for name in [a for a in argv if not a.startswith("--")] or list(CASES):
                fn(name)
            return
    names = [a for a in argv if not a.startswith("--")]
    table = dict(CASES, **LARGE)
    if not names:
        names = list(CASES)
    build_ref_driver()
    for name in names:
        dim, n, k = table[name]
        make_case(name, dim, n, k, histories_only or name in LARGE)


if __name__ == "__main__":
    main(sys.argv[1:])
