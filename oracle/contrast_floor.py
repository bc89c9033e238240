"""Accuracy floor of an FP64 solution for the high-contrast configuration (TEST INFRASTRUCTURE: a
study run on the CPU with the oracle, not part of the product).

Problem: 3D tetrahedral n^3 mesh, HHO k = 2, 4 x 4 x 4 checkerboard coefficient 1 / 1e6, f = 1,
Galerkin coarse operators (the rediscretised hierarchy does not converge at this contrast). For
growing n it reports, with every residual evaluated in extended precision (numpy longdouble):

* floor: ||b - A fl64(x*)|| / ||b|| for x* the exact solution (sparse LU plus iterative refinement
  with extended-precision residuals), rounded to FP64: no FP64 vector does much better;
* oracle: the same for the x the reference's algorithm returns (the oracle restatement of
  FCG(1) + V(1,1) bgs/rbgs in colour order, FlexibleConjugateGradient.h:47-171, stopped by its
  recursive residual at 1e-8, IterativeSolver.h:224-247), and the FP64 evaluation of that residual;
* ratio: || |A| |fl64(x*)| || / ||b||, which scales the FP64 rounding of x into the residual.

Usage: python oracle/contrast_floor.py [n ...]   (default 8 12 16 20)
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as sla

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [ROOT, HERE]

import oracle as O  # noqa: E402
from fhhos4_gb300 import hho  # noqa: E402


def ext_residual(A, b, x):
    """||b - A x|| / ||b|| with the products and sums in extended precision."""
    Al = A.astype(np.longdouble)
    r = np.asarray(b, dtype=np.longdouble) - Al @ np.asarray(x, dtype=np.longdouble)
    return float(np.sqrt(np.sum(r * r)) / np.sqrt(np.sum(np.asarray(b, dtype=np.longdouble) ** 2)))


def study(n: int) -> dict:
    t0 = time.time()
    H = hho.Hierarchy(3, n, 2, coefficient="checkerboard", contrast=1e6, checker_blocks=4, source="one",
                      max_coarse_rows=2000)
    A0 = H.A(0).tocsr()
    Ps = [H.P(l).tocsr() for l in range(H.levels - 1)]
    b = H.b()
    bs = H.block_size
    H.close()
    As = [A0]
    for P in Ps:
        As.append((P.T @ As[-1] @ P).tocsr())
    # exact solution: sparse LU, refined with extended-precision residuals
    lu = sla.splu(A0.tocsc())
    Al = A0.astype(np.longdouble)
    bl = np.asarray(b, dtype=np.longdouble)
    xl = lu.solve(b).astype(np.longdouble)
    for _ in range(4):
        d = lu.solve(np.asarray(bl - Al @ xl, dtype=np.float64))
        xl = xl + d.astype(np.longdouble)
    x64 = np.asarray(xl, dtype=np.float64)
    floor = ext_residual(A0, b, x64)
    ratio = float(np.linalg.norm(abs(A0) @ np.abs(x64)) / np.linalg.norm(b))
    # the reference's algorithm (oracle) in colour order on the Galerkin hierarchy
    perms, _ = O.colour_perms(As, bs)
    Ac, Pc, bc = O.permute_hierarchy(As, Ps, b, bs, perms)
    xo, hist, its, rc = O.fcgmg_solve(Ac, Pc, bc, bs, maxit=400)
    oracle_ext = ext_residual(Ac[0], bc, xo)
    oracle_fp64 = float(np.linalg.norm(bc - Ac[0] @ xo) / np.linalg.norm(bc))
    return dict(n=n, unknowns=A0.shape[0], floor=floor, ratio=ratio, oracle_iterations=its, oracle_status=rc,
                oracle_recursive=float(hist[-1]), oracle_true_ext=oracle_ext, oracle_true_fp64=oracle_fp64,
                seconds=round(time.time() - t0, 1))


def main(argv):
    ns = [int(a) for a in argv] or [8, 12, 16, 20]
    print("n   unknowns   floor(fl64 x*)  ratio |A||x|/|b|  oracle its  recursive   true(ext)   true(FP64 eval)")
    for n in ns:
        r = study(n)
        print(f"{r['n']:<3d} {r['unknowns']:9d}   {r['floor']:.3e}      {r['ratio']:.3e}       {r['oracle_iterations']:4d}"
              f"    {r['oracle_recursive']:.3e}   {r['oracle_true_ext']:.3e}   {r['oracle_true_fp64']:.3e}"
              f"   ({r['seconds']} s)", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
