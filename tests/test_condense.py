"""Static condensation and assembly of the face systems (Diffusion_HHO.h:627-638): the generator's
condensation tables condensed in numpy reproduce its assembled A_0 and b and every rediscretised
coarse operator A_l (which test_generator.py pins against the reference's own), the C ABI validates
the tables before any device call, and the GPU's condensation and assembly give the same CSR
structure and values on every level."""
import numpy as np
import pytest
import scipy.sparse as sp

from fhhos4_gb300 import hho

CASES = [(3, 4, 1), (2, 8, 2), (3, 3, 2), (2, 12, 3)]


def numpy_condense(t):
    """A_0 and b from the condensation tables: per class S = A_FF - A_TF^T A_TT^-1 A_TF and
    G = -A_TF^T A_TT^-1, assembled over the face blocks' two elements."""
    dim, nC, nFF, nI = t["dim"], t["n_cell"], t["n_face_dofs"], t["n_face_blocks"]
    nH, nF = nC + nFF, dim + 1
    nf = nFF // nF
    L = t["local"].reshape(-1, nH, nH)
    Att, Atf, Aff = L[:, :nC, :nC], L[:, :nC, nC:], L[:, nC:, nC:]
    inv = np.linalg.inv(Att)
    S = Aff - np.einsum("cti,ctu,cuj->cij", Atf, inv, Atf)
    G = -np.einsum("cti,ctj->cij", Atf, inv)
    ef = t["elem_faces"].reshape(-1, nF)
    cls = t["elem_class"]
    bT = t["b_cell"].reshape(-1, nC)
    fe = t["face_elems"].reshape(nI, 4)
    rows, cols, vals = [], [], []
    b = np.zeros(nI * nf)
    for I in range(nI):
        for side in range(2):
            e, lfi = fe[I, 2 * side], fe[I, 2 * side + 1]
            c = cls[e]
            for lf in range(nF):
                g = ef[e, lf]
                if g < 0:
                    continue
                blk = S[c][lfi * nf:(lfi + 1) * nf, lf * nf:(lf + 1) * nf]
                r, q = np.meshgrid(np.arange(nf), np.arange(nf), indexing="ij")
                rows.extend((I * nf + r).ravel())
                cols.extend((g * nf + q).ravel())
                vals.extend(blk.ravel())
            b[I * nf:(I + 1) * nf] += G[c][lfi * nf:(lfi + 1) * nf] @ bT[e]
    n = nI * nf
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n)), b


@pytest.mark.parametrize("dim,n,k", CASES[:3])
def test_tables_reproduce_host_assembly(dim, n, k):
    H = hho.Hierarchy(dim, n, k)
    try:
        t = H.condense_tables()
        A0, b0 = H.A(0).tocsr(), H.b()
    finally:
        H.close()
    A, b = numpy_condense(t)
    assert abs(A - A0).max() <= 1e-13 * abs(A0).max()
    assert np.abs(b - b0).max() <= 1e-13 * np.abs(b0).max()


@pytest.mark.parametrize("dim,n,k", [(3, 8, 1), (2, 16, 2)])
def test_level_tables_reproduce_every_level(dim, n, k):
    H = hho.Hierarchy(dim, n, k)
    try:
        for l in range(H.levels):
            A, _ = numpy_condense(H.level_tables(l))
            Al = H.A(l).tocsr()
            assert abs(A - Al).max() <= 1e-13 * abs(Al).max(), l
    finally:
        H.close()


def test_cond_create_validates_tables():
    """Inconsistent tables are refused with FHG_ERR_INVALID_ARG before any device call."""
    from fhhos4_gb300 import _native as N
    H = hho.Hierarchy(2, 4, 1)
    t = H.condense_tables()
    H.close()
    bad = dict(t, face_elems=t["face_elems"].copy())
    bad["face_elems"][1] = (bad["face_elems"][1] + 1) % 3   # the face is not that local face of its element
    with pytest.raises(N.FhgError) as e:
        N.Condense(bad)
    assert e.value.code == N.FHG_ERR_INVALID_ARG and "inconsistent" in str(e.value)
    bad = dict(t, elem_class=t["elem_class"].copy())
    bad["elem_class"][0] = -1
    with pytest.raises(N.FhgError) as e:
        N.Condense(bad)
    assert e.value.code == N.FHG_ERR_INVALID_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("dim,n,k", CASES)
def test_gpu_condensation_matches_host_assembly(dim, n, k):
    from fhhos4_gb300 import _native as N
    H = hho.Hierarchy(dim, n, k)
    try:
        t = H.condense_tables()
        A0, b0 = H.A(0).tocsr(), H.b()
    finally:
        H.close()
    cond = N.Condense(t)
    try:
        nnz, ms = cond.run()
        assert nnz == A0.nnz and ms > 0
        A, b = cond.result(nnz)
        # the same structure (sorted block columns), the values and b to rounding
        assert np.array_equal(A.indptr, A0.indptr) and np.array_equal(A.indices, A0.indices)
        assert np.abs(A.data - A0.data).max() <= 1e-13 * np.abs(A0.data).max()
        assert np.abs(b - b0).max() <= 1e-13 * np.abs(b0).max()
        # a second run gives the same bits
        cond.run()
        A2, b2 = cond.result(nnz)
        assert np.array_equal(A2.data, A.data) and np.array_equal(b2, b)
    finally:
        cond.close()


@pytest.mark.gpu
@pytest.mark.parametrize("dim,n,k", [(3, 16, 1), (2, 32, 2)])
def test_gpu_rediscretisation_of_every_level(dim, n, k):
    """Every level's operator condensed and assembled on the GPU from its element tables: the coarse
    re-discretisation of LevelForHHO::SetupDiscretizedOperator (LevelForHHO.h:72-103)."""
    from fhhos4_gb300 import _native as N
    H = hho.Hierarchy(dim, n, k)
    try:
        for l in range(H.levels):
            Al = H.A(l).tocsr()
            cond = N.Condense(H.level_tables(l))
            try:
                nnz, _ = cond.run()
                A, _ = cond.result(nnz)
            finally:
                cond.close()
            assert np.array_equal(A.indptr, Al.indptr) and np.array_equal(A.indices, Al.indices), l
            assert np.abs(A.data - Al.data).max() <= 1e-13 * np.abs(Al.data).max(), l
    finally:
        H.close()


@pytest.mark.gpu
def test_gpu_condensation_one_class_per_element():
    """Elements not grouped in classes (one local operator per element, as a caller without
    classes passes them): the same system."""
    from fhhos4_gb300 import _native as N
    H = hho.Hierarchy(3, 4, 1)
    try:
        t = H.condense_tables()
        A0 = H.A(0).tocsr()
    finally:
        H.close()
    nH = t["n_cell"] + t["n_face_dofs"]
    local = t["local"].reshape(-1, nH, nH)[t["elem_class"]]
    u = dict(t, n_classes=t["n_elements"], local=local.ravel().copy(),
             elem_class=np.arange(t["n_elements"], dtype=np.int32))
    cond = N.Condense(u)
    try:
        nnz, _ = cond.run()
        A, _ = cond.result(nnz)
        assert np.abs(A.data - A0.data).max() <= 1e-13 * np.abs(A0.data).max()
    finally:
        cond.close()
