"""The tables of P (csrc/hho_gen.cpp, fhg_hho_prolongation_tables): the inputs of assembling
P = Pi_f I_c (LevelForHHO::SetupProlongation_H with CellInterp_Trace, LevelForHHO.h:182-213,
765-954) elsewhere than on the host. A coarse element's contribution to a fine face depends only
on the element's class and on where the face lies in it, so the tables hold one contribution per
such slot and, per fine face, its coarse elements, weights and slots. Assembled here in numpy the
way a table-driven kernel would, they reproduce the generator's P (itself equal to the
reference's to 1e-13): the same structure, the values to rounding (a slot's contribution is
computed at one face of its kind). CPU only."""
import numpy as np
import pytest
import scipy.sparse as sp

from fhhos4_gb300 import hho


def assemble(t, n_coarse_blocks):
    """P from the tables: block row I = sum over its coarse elements t of w_t * contribution[slot_t],
    column block lf of a contribution going to the coarse element's face block lf."""
    bs, nF, nI = t["block_size"], t["faces_per_element"], t["n_face_blocks"]
    rows, cols, vals = [], [], []
    r = np.arange(bs)
    for I in range(nI):
        for s in range(2):
            ce = t["face_ce"][I, s]
            if ce < 0:
                continue
            c = t["face_w"][I, s] * t["slot_contrib"][t["face_slot"][I, s]]
            for lf in range(nF):
                g = t["coarse_elem_faces"][ce, lf]
                if g < 0:
                    continue
                rr, cc = np.meshgrid(I * bs + r, g * bs + r, indexing="ij")
                rows.append(rr.ravel())
                cols.append(cc.ravel())
                vals.append(c[:, lf * bs:(lf + 1) * bs].ravel())
    rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    return sp.csr_matrix((vals, (rows, cols)), shape=(nI * bs, n_coarse_blocks * bs))


@pytest.mark.parametrize("dim,n,k,coefficient", [(2, 16, 1, "identity"), (2, 16, 2, "checkerboard"),
                                                 (3, 8, 1, "identity"), (3, 8, 1, "checkerboard"),
                                                 (3, 4, 2, "identity")])
def test_tables_reproduce_every_prolongation(dim, n, k, coefficient):
    H = hho.Hierarchy(dim, n, k, coefficient=coefficient, contrast=1e3, p_tables=True)
    try:
        for l in range(H.levels - 1):
            t = H.prolongation_tables(l)
            P = H.P(l).tocsr()
            Pt = assemble(t, P.shape[1] // H.block_size)
            # the same block structure (explicit entries included), the values to rounding
            assert np.array_equal(Pt.indptr, P.indptr) and np.array_equal(Pt.indices, P.indices), l
            assert np.abs(Pt.data - P.data).max() <= 1e-13 * np.abs(P.data).max(), l
            # the point of the tables: a number of slots that does not grow with the mesh (280 on the
            # 6-tetrahedra cubes, 44 on the triangle pairs; at most twice that with the two tensors
            # of the checkerboard)
            bound = (280 if dim == 3 else 44) * (2 if coefficient == "checkerboard" else 1)
            assert t["n_slots"] <= bound, (t["n_slots"], t["n_face_blocks"])
            # weights: 1 for a face inside a coarse element, the heterogeneous pair summing to 1 otherwise
            w = np.where(t["face_ce"] >= 0, t["face_w"], 0.0).sum(axis=1)
            assert np.allclose(w, 1.0, rtol=0, atol=1e-15)
    finally:
        H.close()


def test_tables_need_asking_for():
    H = hho.Hierarchy(2, 8, 1, max_levels=2)
    try:
        with pytest.raises(RuntimeError, match="p_tables"):
            H.prolongation_tables(0)
    finally:
        H.close()
