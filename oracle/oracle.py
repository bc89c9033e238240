"""ctypes front end of the CPU restatement in ``oracle/fcgmg_oracle.c``.

TEST INFRASTRUCTURE ONLY. Imported by ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` as the checker; the product never imports it.
Matrices are ``scipy.sparse.csr_matrix`` with int32 indices (the reference's
row-major ``SparseMatrix`` with SMALL_INDEX, src/Utils/Types.h:11-27).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DRIVER = os.path.join(HERE, "_ref", "ref_driver")

BGS_FORWARD, BGS_BACKWARD, BJ, SBGS, ABGS, RABGS = 0, 1, 2, 3, 4, 5
KRYLOV_FCG, KRYLOV_CG = 0, 1
SMOOTHER_CODES = {"bgs": (BGS_FORWARD, 1.0), "rbgs": (BGS_BACKWARD, 1.0),
                  "bj": (BJ, 1.0), "bj23": (BJ, 2.0 / 3.0), "sbgs": (SBGS, 1.0),
                  "abgs": (ABGS, 1.0), "rabgs": (RABGS, 1.0)}
# SmootherFactory.h:37-100: the block SOR codes are the Gauss-Seidel ones (BlockSOR when the
# relaxation parameter is not 1, BlockGaussSeidel when it is).
SOR_ALIASES = {"bsor": "bgs", "rbsor": "rbgs", "sbsor": "sbgs", "absor": "abgs", "rabsor": "rabgs"}


class _CSR(C.Structure):
    _fields_ = [("n_rows", C.c_int), ("n_cols", C.c_int),
                ("rowptr", C.POINTER(C.c_int)), ("colidx", C.POINTER(C.c_int)),
                ("vals", C.POINTER(C.c_double))]


class _Opts(C.Structure):
    _fields_ = [("pre_smoother", C.c_int), ("post_smoother", C.c_int), ("omega", C.c_double),
                ("pre_iterations", C.c_int), ("post_iterations", C.c_int), ("krylov", C.c_int),
                ("tolerance", C.c_double), ("max_iterations", C.c_int), ("w_loops", C.c_int),
                ("coarse_pre_iterations", C.c_int), ("coarse_post_iterations", C.c_int), ("sor_omega", C.c_double)]


_lib = None


def build() -> str:
    """Compile liboracle.so with the oracle Makefile (gcc only)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        srcs = [os.path.join(HERE, f) for f in ("fcgmg_oracle.c", "fcgmg_oracle.h")]
        if not os.path.exists(LIB_PATH) or any(os.path.getmtime(f) > os.path.getmtime(LIB_PATH) for f in srcs):
            build()
        _lib = C.CDLL(LIB_PATH)
    return _lib


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def as_csr(A) -> sp.csr_matrix:
    A = sp.csr_matrix(A)
    A.sort_indices()
    if A.indptr.dtype != np.int32 or A.indices.dtype != np.int32:
        A = sp.csr_matrix((A.data.astype(np.float64), A.indices.astype(np.int32),
                           A.indptr.astype(np.int32)), shape=A.shape)
    A.data = np.ascontiguousarray(A.data, dtype=np.float64)
    return A


def _wrap(A: sp.csr_matrix, keep: list) -> _CSR:
    keep.append(A)
    return _CSR(A.shape[0], A.shape[1], _iptr(A.indptr), _iptr(A.indices), _dptr(A.data))


def spmv(A, x):
    A = as_csr(A); keep = []
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(A.shape[0])
    lib().orc_spmv(C.byref(_wrap(A, keep)), _dptr(x), _dptr(y))
    return y


def residual(A, b, x):
    A = as_csr(A); keep = []
    b = np.ascontiguousarray(b, dtype=np.float64); x = np.ascontiguousarray(x, dtype=np.float64)
    r = np.empty(A.shape[0])
    lib().orc_residual(C.byref(_wrap(A, keep)), _dptr(b), _dptr(x), _dptr(r))
    return r


def spmv_sym_lower(A, x):
    A = as_csr(A); keep = []
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(A.shape[0])
    lib().orc_spmv_sym_lower(C.byref(_wrap(A, keep)), _dptr(x), _dptr(y))
    return y


def block_gs(A, bs, b, x, backward=False):
    A = as_csr(A); keep = []
    x = np.array(x, dtype=np.float64, copy=True)
    b = np.ascontiguousarray(b, dtype=np.float64)
    lib().orc_block_gs(C.byref(_wrap(A, keep)), C.c_int(bs), _dptr(b), _dptr(x), C.c_int(int(backward)))
    return x


def block_jacobi(A, bs, omega, b, x):
    A = as_csr(A); keep = []
    x = np.array(x, dtype=np.float64, copy=True)
    b = np.ascontiguousarray(b, dtype=np.float64)
    lib().orc_block_jacobi(C.byref(_wrap(A, keep)), C.c_int(bs), C.c_double(omega), _dptr(b), _dptr(x))
    return x


def greedy_colouring(A, bs):
    """Colour of every block row and the colour count."""
    A = as_csr(A); keep = []
    nb = A.shape[0] // bs
    colour = np.empty(nb, dtype=np.int32)
    nc = lib().orc_greedy_colouring(C.byref(_wrap(A, keep)), C.c_int(bs), _iptr(colour))
    return colour, int(nc)


def colour_permutation(colour, ncolours):
    """perm[new_block] = old_block, block rows grouped by ascending colour."""
    colour = np.ascontiguousarray(colour, dtype=np.int32)
    perm = np.empty(len(colour), dtype=np.int32)
    lib().orc_colour_permutation(C.c_int(len(colour)), _iptr(colour), C.c_int(ncolours), _iptr(perm))
    return perm


def set_threads(n: int):
    lib().orc_set_threads(C.c_int(n))


def max_threads() -> int:
    return int(lib().orc_max_threads())


def last_timing():
    """(setup seconds, iteration seconds) of the last fcgmg_solve."""
    s, i = C.c_double(), C.c_double()
    lib().orc_last_timing(C.byref(s), C.byref(i))
    return s.value, i.value


def fcgmg_solve(As, Ps, b, bs, pre="bgs", post="rbgs", krylov="fcg", tol=1e-8, maxit=200,
                pre_iterations=1, post_iterations=1, cycle="V", coarse_iterations=(-1, -1), omega=1.0):
    """Returns (x, history, iterations, status). bs: the block size, or one per level (a p-multigrid
    hierarchy, whose P between face degrees is the natural injection). coarse_iterations: smoothing
    steps on levels >= 1 (-1: those of level 0, the reference's behaviour). omega: Multigrid::RelaxationParameter, the
    relaxation of "bj" and, when not 1, block SOR in place of the Gauss-Seidel codes
    (SmootherFactory.h:37-100); "bj23" keeps 2/3."""
    keep: list = []
    nl = len(As)
    Aarr = (_CSR * nl)(*[_wrap(as_csr(A), keep) for A in As])
    Parr = (_CSR * max(nl - 1, 1))(*([_wrap(as_csr(P), keep) for P in Ps] or [_CSR()]))
    pre, post = SOR_ALIASES.get(pre, pre), SOR_ALIASES.get(post, post)
    pc, om = SMOOTHER_CODES[pre]
    qc, om2 = SMOOTHER_CODES[post]
    jac = om if pc == BJ else om2
    if (pre == "bj" or post == "bj") and "bj23" not in (pre, post):
        jac = omega
    opts = _Opts(pc, qc, jac, pre_iterations, post_iterations,
                 KRYLOV_CG if krylov == "cg" else KRYLOV_FCG, tol, maxit,
                 2 if cycle == "W" else (-1 if cycle == "K" else 1), int(coarse_iterations[0]),
                 int(coarse_iterations[1]), float(omega))
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(As[0].shape[0])
    hist = np.zeros(maxit + 1)
    iters = C.c_int(0)
    bs_l = np.ascontiguousarray(np.broadcast_to(np.asarray(bs, dtype=np.int32), (nl,)), dtype=np.int32)
    rc = lib().orc_fcgmg_solve_levels(C.c_int(nl), _iptr(bs_l), Aarr, Parr, _dptr(b), _dptr(x),
                               C.byref(opts), _dptr(hist), C.byref(iters))
    return x, hist[: iters.value + 1].copy(), iters.value, rc


def permute_hierarchy(As, Ps, b, bs, perms):
    """Block-permute a hierarchy: A'_l = Pi_l A_l Pi_l^T, P'_l = Pi_l P_l Pi_{l+1}^T, b' = Pi_0 b.

    perms[l][new_block] = old_block on level l; bs: the block size, or one per level.
    """
    bs_l = np.broadcast_to(np.asarray(bs), (len(As),))

    def scalar_perm(pb, b):
        return (pb[:, None] * b + np.arange(b)[None, :]).ravel()

    sps = [scalar_perm(np.asarray(p), int(b)) for p, b in zip(perms, bs_l)]
    As2 = [as_csr(as_csr(A)[s][:, s]) for A, s in zip(As, sps)]
    Ps2 = [as_csr(as_csr(P)[sps[l]][:, sps[l + 1]]) for l, P in enumerate(Ps)]
    return As2, Ps2, np.asarray(b)[sps[0]]


def colour_perms(As, bs):
    """Greedy-colouring block permutation of every level (the coarsest stays natural); bs: the block
    size, or one per level."""
    perms, ncol = [], []
    bs_l = np.broadcast_to(np.asarray(bs), (len(As),))
    for l, A in enumerate(As):
        b = int(bs_l[l])
        nb = A.shape[0] // b
        if l == len(As) - 1:
            perms.append(np.arange(nb, dtype=np.int32)); ncol.append(0)
            continue
        c, nc = greedy_colouring(A, b)
        perms.append(colour_permutation(c, nc)); ncol.append(nc)
    return perms, ncol
