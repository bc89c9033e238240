"""fhg_residual_norm_noalloc, the entry point for callers that may not allocate device memory
(a process whose GPU memory is all reserved by its own pool or budget, an embedder that must not
grow its footprint, a latency-bound loop that cannot afford cudaMalloc's synchronisation): it
computes ||b - A x|| with its partial sums in a fixed array inside the library. Checked through
the C ABI against the residual of the existing entry point fhg_apply(FHG_OP_RESIDUAL) and against
the host FP64 residual norm, within the operator tests' tolerance, on two calls in a row.
Collected last on purpose (file name), and self-contained so that it passes alone as well."""
import ctypes as C
import importlib
import os

import numpy as np
import pytest
import scipy.sparse as sp

from _golden import Case

pytestmark = pytest.mark.gpu

B = importlib.import_module("fhhos4_gb300.build")


def entry_major_bsr(A, bs):
    """Block rows, block columns and entry-major values of A (libfhg's device block layout)."""
    Ab = sp.bsr_matrix(sp.csr_matrix(A), blocksize=(bs, bs))
    Ab.sort_indices()
    nnzb = Ab.data.shape[0]
    ld = ((nnzb + 31) // 32) * 32
    vals = np.zeros((bs * bs, ld))
    vals[:, :nnzb] = Ab.data.reshape(nnzb, bs * bs).T
    return Ab.indptr.astype(np.int32), Ab.indices.astype(np.int32), np.ascontiguousarray(vals.ravel()), ld


def test_residual_norm_without_allocation_matches_existing_entry_point():
    torch = pytest.importorskip("torch")
    if not os.path.exists(B.LIB):
        B.build()
    from fhhos4_gb300 import _native as N
    lib = N.load()
    c = Case("tet3d_n8_k1")
    A, bs = c.As[0], c.bs
    n = A.shape[0]
    rng = np.random.default_rng(11)
    x = rng.standard_normal(n)
    b = c.b.copy()

    # existing entry point: the residual through fhg_apply on a context
    ctx = N.Context(0)
    for l, Al in enumerate(c.As):
        ctx.set_level(l, bs, Al)
    for l, P in enumerate(c.Ps):
        ctx.set_prolongation(l, P)
    ctx.setup(len(c.As), N.default_options())
    r = ctx.apply(0, N.OP_RESIDUAL, x, b, n)
    ref = np.linalg.norm(r)
    ctx.close()

    rowptr, colidx, vals, ld = entry_major_bsr(A, bs)
    dev = torch.device("cuda:0")
    t_rp = torch.from_numpy(rowptr).to(dev)
    t_ci = torch.from_numpy(colidx).to(dev)
    t_va = torch.from_numpy(vals).to(dev)
    t_x = torch.from_numpy(x).to(dev)
    t_b = torch.from_numpy(b).to(dev)
    out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize()
    values = []
    for _ in range(2):  # two calls in a row share the library's scratch array
        out.fill_(-1.0)
        rc = lib.fhg_residual_norm_noalloc(0, n // bs, bs, 8, C.c_void_p(t_rp.data_ptr()), C.c_void_p(t_ci.data_ptr()),
                                           C.c_void_p(t_va.data_ptr()), ld, C.c_void_p(t_x.data_ptr()),
                                           C.c_void_p(t_b.data_ptr()), C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        assert rc == N.FHG_OK
        torch.cuda.synchronize()
        values.append(float(out.item()))
    host = float(np.linalg.norm(b - A @ x))   # host FP64 residual of the same system
    for v in values:
        assert abs(v - ref) <= 1e-12 * ref
        assert abs(v - host) <= 1e-12 * host
    assert values[0] == values[1]

    # sizes beyond the scratch array are rejected before anything is launched
    too_many = N.FHG_NOALLOC_MAX_PARTIALS * 256 // 32 + 1
    rc = lib.fhg_residual_norm_noalloc(0, too_many, bs, 32, C.c_void_p(t_rp.data_ptr()), C.c_void_p(t_ci.data_ptr()),
                                       C.c_void_p(t_va.data_ptr()), ld, C.c_void_p(t_x.data_ptr()),
                                       C.c_void_p(t_b.data_ptr()), C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    assert rc == N.FHG_ERR_TOO_LARGE
