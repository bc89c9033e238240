"""Post-processing of a face solution (cell-unknown recovery, k+1 reconstruction, L2 error;
Diffusion_HHO.h:855-912 and :120-150): the generator's element tables evaluated in numpy reproduce
the host L2 error (which test_generator.py pins against the reference's own L2Error), the C ABI
validates its tables before any device call, and the GPU pass gives the host's cell unknowns and
L2 error."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse.linalg as sla

from fhhos4_gb300 import hho

CASES = [(3, 6, 1), (2, 16, 2), (3, 4, 2)]


def _solved(dim, n, k):
    H = hho.Hierarchy(dim, n, k)
    x = sla.spsolve(H.A(0).tocsc(), H.b())
    return H, x


def numpy_post(t, x):
    """Cell unknowns and relative L2 error of the reconstruction from the element tables."""
    dim, ne, nC, nFF, nR, nq = (t[k] for k in ("dim", "n_elements", "n_cell", "n_face_dofs", "n_recon", "n_points"))
    nF = dim + 1
    nf = nFF // nF
    cls = t["elem_class"]
    faces = t["elem_faces"].reshape(ne, nF)
    xf = np.zeros((ne, nFF))
    xb = x.reshape(-1, nf)
    for lf in range(nF):
        g = faces[:, lf]
        m = g >= 0
        xf[m, lf * nf:(lf + 1) * nf] = xb[g[m]]
    xc = t["cell_rhs"].reshape(ne, nC) + np.einsum("eij,ej->ei", t["solve_cells"].reshape(-1, nC, nFF)[cls], xf)
    coef = np.einsum("eij,ej->ei", t["recon"].reshape(-1, nR, nC + nFF)[cls], np.concatenate([xc, xf], 1))
    uh = np.einsum("eqi,ei->eq", t["basis"].reshape(-1, nq, nR)[cls], coef)
    X = t["elem_centre"].reshape(ne, 3)[:, None, :] + t["offsets"].reshape(-1, nq, 3)[cls]
    u = np.prod(np.sin(np.pi * X[:, :, :dim]), axis=2)
    W = t["weights"].reshape(-1, nq)[cls]
    return xc, float(np.sqrt((W * (uh - u) ** 2).sum()) / np.sqrt((W * u * u).sum()))


@pytest.mark.parametrize("dim,n,k", CASES)
def test_tables_reproduce_host_l2_error(dim, n, k):
    H, x = _solved(dim, n, k)
    try:
        t = H.post_tables()
        assert t["n_classes"] < t["n_elements"]   # translated elements share their tables
        _, err = numpy_post(t, x)
        assert err == pytest.approx(H.l2_error(x), rel=1e-11)
    finally:
        H.close()


def test_post_create_validates_tables():
    """Bad tables are refused with FHG_ERR_INVALID_ARG / FHG_ERR_UNSUPPORTED before any device call."""
    from fhhos4_gb300 import _native as N
    H = hho.Hierarchy(2, 4, 1)
    t = H.post_tables()
    H.close()
    bad = dict(t)
    bad["elem_class"] = t["elem_class"].copy()
    bad["elem_class"][3] = t["n_classes"]
    with pytest.raises(N.FhgError) as e:
        N.Post(bad)
    assert e.value.code == N.FHG_ERR_INVALID_ARG and "class" in str(e.value)
    big = dict(t, n_points=100000)
    with pytest.raises(N.FhgError) as e:
        N.Post(big)
    assert e.value.code == N.FHG_ERR_UNSUPPORTED


@pytest.mark.gpu
@pytest.mark.parametrize("dim,n,k", CASES)
def test_gpu_post_matches_host(dim, n, k):
    import torch
    from fhhos4_gb300 import _native as N
    H, x = _solved(dim, n, k)
    try:
        t = H.post_tables()
        host_err = H.l2_error(x)
    finally:
        H.close()
    xc_ref, _ = numpy_post(t, x)
    post = N.Post(t)
    try:
        xd = torch.tensor(x, device="cuda")
        cells = torch.zeros(t["n_elements"] * t["n_cell"], dtype=torch.float64, device="cuda")
        err, ms = post.run(xd.data_ptr(), cells.data_ptr(), "sine")
        assert ms > 0
        assert err == pytest.approx(host_err, rel=1e-11)
        xc = cells.cpu().numpy().reshape(xc_ref.shape)
        assert np.abs(xc - xc_ref).max() <= 1e-12 * np.abs(xc_ref).max()
        # cell unknowns only
        cells.zero_()
        none, _ = post.run(xd.data_ptr(), cells.data_ptr(), "none")
        assert none is None
        assert np.abs(cells.cpu().numpy().reshape(xc_ref.shape) - xc).max() == 0.0
        # the same launch twice: the fixed-order reduction gives the same bits
        err2, _ = post.run(xd.data_ptr(), 0, "sine")
        assert err2 == err
    finally:
        post.close()


@pytest.mark.gpu
def test_gpu_post_of_gpu_solve():
    """The whole path on the device: FCG + V-cycle solve of the 3D sine problem, then its L2 error,
    equal to the host's evaluation of the same x."""
    import torch
    from fhhos4_gb300 import _native as N
    from fhhos4_gb300 import solver as S
    H = hho.Hierarchy(3, 8, 1)
    try:
        As = [H.A(l) for l in range(H.levels)]
        Ps = [H.P(l) for l in range(H.levels - 1)]
        b = H.b()
        s = S.fcg_mg(As, Ps, H.block_size, precision="fp32")
        x = s.Solve(b)
        t = H.post_tables()
        host_err = H.l2_error(x)
    finally:
        H.close()
    post = N.Post(t)
    try:
        err, _ = post.run(torch.tensor(x, device="cuda").data_ptr(), 0, "sine")
        assert err == pytest.approx(host_err, rel=1e-11)
        assert 1e-4 < err < 1e-2   # the discretisation error of 8^3, k = 1
    finally:
        post.close()
