"""libfhg's host-side setup algebra (fhhos4_gb300/csrc/fhg_host.h, the code fhg_setup runs before
anything goes to the GPU) on the CPU, through oracle/host_check.cpp: the greedy colouring against
the oracle's (bit-exact, on the reference's hierarchies), the natural-injection test and its
Galerkin operator against scipy (exact), the block Galerkin product R A P (1e-14), the symmetrised
outer operator (exact), and the block and dense inverses against numpy."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

import oracle as O
from _golden import FULL_CASES, Case, available

from fhhos4_gb300 import hho

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_build", "libhostcheck.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "hostcheck"], check=True, timeout=300)
        _lib = C.CDLL(LIB)
        _lib.hc_inject_galerkin.restype = C.c_longlong
        _lib.hc_galerkin.restype = C.c_longlong
        _lib.hc_symmetrise_lower.restype = C.c_longlong
    return _lib


def ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def csr(A):
    A = sp.csr_matrix(A)
    A.sort_indices()
    return (np.ascontiguousarray(A.indptr, dtype=np.int32), np.ascontiguousarray(A.indices, dtype=np.int32),
            np.ascontiguousarray(A.data, dtype=np.float64))


def call_matrix(fn, rows, cap):
    """Run a hc_* producer of a square CSR matrix of `rows` rows (capacity protocol: called again
    with the reported entry count when `cap` was too small); returns it as a csr_matrix."""
    while True:
        n = C.c_int()
        rp = np.zeros(rows + 1, dtype=np.int32)
        ci = np.zeros(max(cap, 1), dtype=np.int32)
        va = np.zeros(max(cap, 1), dtype=np.float64)
        nnz = fn(C.byref(n), ip(rp), ip(ci), dp(va), C.c_longlong(cap))
        if nnz <= cap:
            assert n.value == rows
            return sp.csr_matrix((va[:nnz], ci[:nnz], rp), shape=(rows, rows))
        cap = int(nnz)


@pytest.fixture(scope="module", params=available(FULL_CASES))
def case(request):
    return Case(request.param)


def test_colouring_is_the_oracles(case):
    """The colouring fhg_setup computes is the oracle's, bit for bit, on every level (the GPU
    tests compare the permutations it leads to)."""
    for l, A in enumerate(case.As[:-1]):
        rp, ci, va = csr(A)
        colour = np.empty(A.shape[0] // case.bs, dtype=np.int32)
        nc = lib().hc_colouring(A.shape[0], ip(rp), ip(ci), dp(va), case.bs, ip(colour))
        ref, nref = O.greedy_colouring(A, case.bs)
        assert nc == nref and np.array_equal(colour, ref), l


def test_symmetrised_outer_operator(case):
    A = case.As[0]
    rp, ci, va = csr(A)
    n = A.shape[0]
    cap = 2 * A.nnz
    orp, oci, ova = np.zeros(n + 1, np.int32), np.zeros(cap, np.int32), np.zeros(cap)
    nnz = lib().hc_symmetrise_lower(n, ip(rp), ip(ci), dp(va), ip(orp), ip(oci), dp(ova), C.c_longlong(cap))
    S = sp.csr_matrix((ova[:nnz], oci[:nnz], orp), shape=A.shape)
    ref = sp.tril(A) + sp.tril(A, -1).T
    assert abs(S - ref).max() == 0.0


def test_block_galerkin_product(case):
    """R A P with R = P^T by the block products of the Galerkin setup, against scipy."""
    if case.levels < 2:
        pytest.skip("a single level: no prolongation")
    A, P = case.As[0], case.Ps[0]
    arp, aci, ava = csr(A)
    prp, pci, pva = csr(P)
    fn = lambda *a: lib().hc_galerkin(A.shape[0], ip(arp), ip(aci), dp(ava), P.shape[1], ip(prp), ip(pci), dp(pva),
                                      case.bs, *a)
    G = call_matrix(fn, P.shape[1], case.As[1].nnz // 2)   # too small at first: exercises the retry
    ref = (P.T @ A @ P).tocsr()
    assert abs(G - ref).max() <= 1e-14 * abs(ref).max()


@pytest.mark.parametrize("dim,n,k", [(2, 16, 3), (3, 4, 2)])
def test_natural_injection_and_its_galerkin_operator(dim, n, k):
    As, Ps, b, bss, _ = hho.generate_p(dim, n, k, "ch")
    A, P = As[0], Ps[0]
    nh, nl = bss[0], bss[1]
    prp, pci, pva = csr(P)
    assert lib().hc_natural_injection(P.shape[0], P.shape[1], ip(prp), ip(pci), dp(pva), nh) == nl
    # anything else is not the injection: another value, another column, an extra entry, an h-transfer
    bad = pva.copy(); bad[3] = 0.5
    assert lib().hc_natural_injection(P.shape[0], P.shape[1], ip(prp), ip(pci), dp(bad), nh) == 0
    badc = pci.copy(); badc[3] += 1
    assert lib().hc_natural_injection(P.shape[0], P.shape[1], ip(prp), ip(badc), dp(pva), nh) == 0
    Q = P.tolil(); Q[nl, 0] = 1.0
    qrp, qci, qva = csr(Q.tocsr())
    assert lib().hc_natural_injection(P.shape[0], P.shape[1], ip(qrp), ip(qci), dp(qva), nh) == 0
    H = hho.Hierarchy(dim, n, 1)
    Ph = H.P(0)
    H.close()
    hrp, hci, hva = csr(Ph)
    assert lib().hc_natural_injection(Ph.shape[0], Ph.shape[1], ip(hrp), ip(hci), dp(hva), nl) == 0
    # P^T A P over the injection: the leading block of every block, the entries as they are
    arp, aci, ava = csr(A)
    fn = lambda *a: lib().hc_inject_galerkin(A.shape[0], ip(arp), ip(aci), dp(ava), nh, nl, *a)
    G = call_matrix(fn, P.shape[1], A.nnz)
    ref = (P.T @ A @ P).tocsr()
    assert abs(G - ref).max() == 0.0


@pytest.mark.parametrize("n", [2, 3, 4, 6])
def test_block_inverse(n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n)) + n * np.eye(n)
    inv = np.zeros((n, n))
    assert lib().hc_invert_block(dp(np.ascontiguousarray(a)), n, dp(inv)) == 1
    assert np.abs(inv - np.linalg.inv(a)).max() <= 1e-13 * np.abs(np.linalg.inv(a)).max()
    assert lib().hc_invert_block(dp(np.zeros((n, n))), n, dp(inv)) == 0


def test_dense_spd_inverse():
    rng = np.random.default_rng(5)
    m = rng.standard_normal((300, 300))
    a = m @ m.T + 300 * np.eye(300)
    inv = np.zeros_like(a)
    assert lib().hc_dense_spd_inverse(dp(np.ascontiguousarray(a)), 300, dp(inv)) == 0
    ref = np.linalg.inv(a)
    assert np.abs(inv - ref).max() <= 1e-12 * np.abs(ref).max()
    neg = -a
    assert lib().hc_dense_spd_inverse(dp(np.ascontiguousarray(neg)), 300, dp(inv)) != 0
