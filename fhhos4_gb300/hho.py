"""ctypes front end of the host hierarchy producer (csrc/hho_gen.cpp, libfhg_hho.so).

``generate(dim, n, k, ...)`` returns the condensed HHO face operators ``As``, prolongations
``Ps``, right-hand side ``b`` and block size of fhhos4's geometric multigrid hierarchy on the
in-house unit-square (2 triangles per cell) or unit-cube (6 tetrahedra per cube) mesh.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import scipy.sparse as sp

from .build import HHO_LIB

SOURCE = {"sine": 0, "one": 1, "modes": 2}
COEFFICIENT = {"identity": 0, "checkerboard": 1, "anisotropic": 2, "lognormal_patches": 3}


class Params(C.Structure):
    _fields_ = [("dim", C.c_int), ("n", C.c_int), ("k", C.c_int), ("max_coarse_rows", C.c_int),
                ("max_levels", C.c_int), ("source", C.c_int), ("coefficient", C.c_int), ("contrast", C.c_double),
                ("checker_blocks", C.c_int), ("threads", C.c_int), ("eps_min", C.c_double),
                ("seed", C.c_ulonglong), ("p_tables", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(HHO_LIB):
            raise ImportError(f"{HHO_LIB} is missing: build it with `python -m fhhos4_gb300.build`")
        L = C.CDLL(HHO_LIB)
        P = C.POINTER
        L.fhg_hho_default_params.argtypes = [P(Params)]
        L.fhg_hho_create.argtypes = [P(C.c_void_p), P(Params)]
        L.fhg_hho_destroy.argtypes = [C.c_void_p]
        L.fhg_hho_last_error.argtypes = [C.c_void_p]
        L.fhg_hho_last_error.restype = C.c_char_p
        L.fhg_hho_num_levels.argtypes = [C.c_void_p]
        L.fhg_hho_block_size.argtypes = [C.c_void_p]
        L.fhg_hho_level.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_longlong), P(P(C.c_int)),
                                    P(P(C.c_int)), P(P(C.c_double))]
        L.fhg_hho_prolongation.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_int), P(C.c_longlong),
                                           P(P(C.c_int)), P(P(C.c_int)), P(P(C.c_double))]
        L.fhg_hho_rhs.argtypes = [C.c_void_p, P(P(C.c_double))]
        L.fhg_hho_l2_error.argtypes = [C.c_void_p, C.c_void_p, P(C.c_double)]
        L.fhg_hho_face_tensors.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.fhg_hho_post_sizes.argtypes = [C.c_void_p] + [P(C.c_int)] * 6
        L.fhg_hho_post_tables.argtypes = [C.c_void_p] + [C.c_void_p] * 9
        L.fhg_hho_condense_tables.argtypes = [C.c_void_p] + [C.c_void_p] * 3
        L.fhg_hho_level_sizes.argtypes = [C.c_void_p, C.c_int] + [P(C.c_int)] * 5
        L.fhg_hho_level_tables.argtypes = [C.c_void_p, C.c_int] + [C.c_void_p] * 4
        _lib = L
    return _lib


def _arr(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class Hierarchy:
    """Owns one generated hierarchy; arrays are copied out into numpy."""

    def __init__(self, dim: int, n: int, k: int = 1, max_coarse_rows: int = 1000, max_levels: int = 0,
                 source: str = "sine", coefficient: str = "identity", contrast: float = 1.0, checker_blocks: int = 4,
                 threads: int = 0, eps_min: float = 1e-3, seed: int = 20261203, p_tables: bool = False):
        L = lib()
        p = Params()
        L.fhg_hho_default_params(C.byref(p))
        p.dim, p.n, p.k = dim, n, k
        p.max_coarse_rows, p.max_levels = max_coarse_rows, max_levels
        p.source, p.coefficient = SOURCE[source], COEFFICIENT[coefficient]
        p.contrast, p.checker_blocks, p.threads = contrast, checker_blocks, threads
        p.eps_min, p.seed = eps_min, seed
        p.p_tables = 1 if p_tables else 0
        self.h = C.c_void_p()
        self.dim = dim
        rc = L.fhg_hho_create(C.byref(self.h), C.byref(p))
        if rc != 0:
            msg = L.fhg_hho_last_error(self.h).decode()
            L.fhg_hho_destroy(self.h)
            raise RuntimeError(f"hierarchy generation failed: {msg}")
        self.levels = L.fhg_hho_num_levels(self.h)
        self.block_size = L.fhg_hho_block_size(self.h)

    def A(self, l: int) -> sp.csr_matrix:
        L = lib()
        n, nnz = C.c_int(), C.c_longlong()
        rp, ci, va = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_double)()
        L.fhg_hho_level(self.h, l, C.byref(n), C.byref(nnz), C.byref(rp), C.byref(ci), C.byref(va))
        return sp.csr_matrix((_arr(va, nnz.value, np.float64), _arr(ci, nnz.value, np.int32),
                              _arr(rp, n.value + 1, np.int32)), shape=(n.value, n.value))

    def P(self, l: int) -> sp.csr_matrix:
        L = lib()
        nr, nc, nnz = C.c_int(), C.c_int(), C.c_longlong()
        rp, ci, va = C.POINTER(C.c_int)(), C.POINTER(C.c_int)(), C.POINTER(C.c_double)()
        L.fhg_hho_prolongation(self.h, l, C.byref(nr), C.byref(nc), C.byref(nnz), C.byref(rp), C.byref(ci),
                               C.byref(va))
        return sp.csr_matrix((_arr(va, nnz.value, np.float64), _arr(ci, nnz.value, np.int32),
                              _arr(rp, nr.value + 1, np.int32)), shape=(nr.value, nc.value))

    def prolongation_tables(self, l: int) -> dict:
        """The tables of P_l (the hierarchy made with p_tables=True): per unknown fine face its coarse
        elements `face_ce` (n, 2; -1: none), weights `face_w` and slots `face_slot`; per slot the
        contribution `slot_contrib` (bs x faces_per_element*bs); per coarse element its unknown face
        blocks `coarse_elem_faces` (-1: Dirichlet)."""
        L = lib()
        sz = [C.c_int() for _ in range(5)]
        rc = L.fhg_hho_prolongation_table_sizes(self.h, l, *[C.byref(v) for v in sz])
        if rc != 0:
            raise RuntimeError("no prolongation tables (make the hierarchy with p_tables=True)" if rc == -2
                               else "prolongation_table_sizes failed")
        nI, ns, nce, bs, nF = (v.value for v in sz)
        t = dict(n_face_blocks=nI, n_slots=ns, n_coarse_elements=nce, block_size=bs, faces_per_element=nF,
                 face_ce=np.zeros((nI, 2), np.int32), face_w=np.zeros((nI, 2)), face_slot=np.zeros((nI, 2), np.int32),
                 slot_contrib=np.zeros((ns, bs, nF * bs)), coarse_elem_faces=np.zeros((nce, nF), np.int32))
        if L.fhg_hho_prolongation_tables(self.h, l, *[C.c_void_p(t[k].ctypes.data) for k in
                                                      ("face_ce", "face_w", "face_slot", "slot_contrib",
                                                       "coarse_elem_faces")]) != 0:
            raise RuntimeError("prolongation_tables failed")
        return t

    def b(self) -> np.ndarray:
        L = lib()
        p = C.POINTER(C.c_double)()
        L.fhg_hho_rhs(self.h, C.byref(p))
        n = self.A_rows(0)
        return _arr(p, n, np.float64)

    def l2_error(self, x) -> float:
        """Relative L2 error of the k+1 reconstruction of face solution x against the exact solution
        (sine source only), as the reference's Diffusion_HHO::L2Error."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = C.c_double()
        rc = lib().fhg_hho_l2_error(self.h, C.c_void_p(x.ctypes.data), C.byref(out))
        if rc != 0:
            raise RuntimeError("no exact solution for this source" if rc == -2 else "l2_error failed")
        return out.value

    def face_tensors(self, l: int = 0) -> np.ndarray:
        """(n_blocks, 12): diffusion tensors of the two elements of every unknown face of level l,
        (xx, yy, zz, xy, xz, yz) each in 3D, (xx, yy, xy, 0, 0, 0) in 2D."""
        nb = self.A_rows(l) // self.block_size
        out = np.zeros((nb, 12), dtype=np.float64)
        if lib().fhg_hho_face_tensors(self.h, l, C.c_void_p(out.ctypes.data)) != 0:
            raise RuntimeError("face_tensors failed")
        return out

    def post_tables(self) -> dict:
        """The finest level's element tables for post-processing (cell-unknown recovery and the L2 error
        of the reconstruction; fhg_post_create takes them): sizes and arrays."""
        sz = [C.c_int() for _ in range(6)]
        if lib().fhg_hho_post_sizes(self.h, *[C.byref(v) for v in sz]) != 0:
            raise RuntimeError("post_sizes failed")
        ne, ncls, nC, nFF, nR, nq = (v.value for v in sz)
        dim = self.dim
        nF = dim + 1
        t = dict(dim=dim, n_elements=ne, n_classes=ncls, n_cell=nC, n_face_dofs=nFF, n_recon=nR, n_points=nq,
                 elem_class=np.zeros(ne, np.int32), elem_faces=np.zeros(ne * nF, np.int32),
                 elem_centre=np.zeros(ne * 3), cell_rhs=np.zeros(ne * nC), solve_cells=np.zeros(ncls * nC * nFF),
                 recon=np.zeros(ncls * nR * (nC + nFF)), weights=np.zeros(ncls * nq), offsets=np.zeros(ncls * nq * 3),
                 basis=np.zeros(ncls * nq * nR))
        names = ["elem_class", "elem_faces", "elem_centre", "cell_rhs", "solve_cells", "recon", "weights", "offsets",
                 "basis"]
        if lib().fhg_hho_post_tables(self.h, *[C.c_void_p(t[k].ctypes.data) for k in names]) != 0:
            raise RuntimeError("post_tables failed")
        return t

    def condense_tables(self) -> dict:
        """The finest level's inputs of static condensation (fhg_cond_create takes them): the post
        tables' element classes and faces, per class the local operator before condensation, per
        element b_T, per unknown face block its two elements and local face indices."""
        t = self.post_tables()
        nH = t["n_cell"] + t["n_face_dofs"]
        nI = self.A_rows(0) // self.block_size
        t.update(n_face_blocks=nI, local=np.zeros(t["n_classes"] * nH * nH),
                 b_cell=np.zeros(t["n_elements"] * t["n_cell"]), face_elems=np.zeros(nI * 4, np.int32))
        if lib().fhg_hho_condense_tables(self.h, C.c_void_p(t["local"].ctypes.data), C.c_void_p(t["b_cell"].ctypes.data),
                                         C.c_void_p(t["face_elems"].ctypes.data)) != 0:
            raise RuntimeError("condense_tables failed")
        return t

    def level_tables(self, l: int) -> dict:
        """Condensation inputs of level l (fhg_cond_create takes them; no source term, b_cell = 0)."""
        sz = [C.c_int() for _ in range(5)]
        if lib().fhg_hho_level_sizes(self.h, l, *[C.byref(v) for v in sz]) != 0:
            raise RuntimeError("level_sizes failed")
        ne, ncls, nC, nFF, nI = (v.value for v in sz)
        nH, nF = nC + nFF, self.dim + 1
        t = dict(dim=self.dim, n_elements=ne, n_classes=ncls, n_cell=nC, n_face_dofs=nFF, n_face_blocks=nI,
                 elem_class=np.zeros(ne, np.int32), elem_faces=np.zeros(ne * nF, np.int32),
                 local=np.zeros(ncls * nH * nH), face_elems=np.zeros(nI * 4, np.int32), b_cell=np.zeros(ne * nC))
        if lib().fhg_hho_level_tables(self.h, l, *[C.c_void_p(t[k].ctypes.data)
                                                   for k in ("elem_class", "elem_faces", "local", "face_elems")]) != 0:
            raise RuntimeError("level_tables failed")
        return t

    def A_rows(self, l: int) -> int:
        n = C.c_int()
        lib().fhg_hho_level(self.h, l, C.byref(n), None, None, None, None)
        return n.value

    def close(self):
        if self.h:
            lib().fhg_hho_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def generate(dim: int, n: int, k: int = 1, **kw):
    """(As, Ps, b, block_size) of the hierarchy."""
    H = Hierarchy(dim, n, k, **kw)
    As = [H.A(l) for l in range(H.levels)]
    Ps = [H.P(l) for l in range(H.levels - 1)]
    b = H.b()
    bs = H.block_size
    H.close()
    return As, Ps, b, bs


# ---------------------------------------------------------------------------
# p-multigrid hierarchy (src/Solver/Multigrid/MultigridForHHO/P_MultigridForHHO.h)

P_STRATEGIES = ("minus1", "minus2", "divide_by_2", "direct_to_low")


def face_unknowns(dim: int, k: int) -> int:
    """Face-basis functions of degree k (HHOParameters::nFaceUnknowns): k + 1 on edges, (k+1)(k+2)/2
    on triangles."""
    return k + 1 if dim == 2 else (k + 1) * (k + 2) // 2


def natural_injection(n_faces: int, nh: int, nl: int) -> sp.csr_matrix:
    """P_LevelForHHO::SetupProlongation (P_MultigridForHHO.h:69-92): on every face the nl functions of
    the lower degree are the first nl of the nh of the higher one (hierarchical face bases), so P
    holds a 1 at (f * nh + i, f * nl + i) for i < nl; R = P^T (P_MultigridForHHO.h:95-98)."""
    f = np.arange(n_faces)[:, None]
    i = np.arange(nl)[None, :]
    rows, cols = (f * nh + i).ravel(), (f * nl + i).ravel()
    return sp.csr_matrix((np.ones(rows.size), (rows, cols)), shape=(n_faces * nh, n_faces * nl))


def p_degrees(dim: int, k: int, n_faces: int, strategy: str = "minus2", coarse_poly_degree: int = 1,
              max_coarse_rows: int = 1000):
    """Face degrees of the levels Multigrid::Setup creates with HP_CoarsStgy::P_only
    (src/Solver/Multigrid/Multigrid.h:121-224, 353-361, 419-427): from k, a new level while the
    current one has more than max_coarse_rows unknowns and a degree above coarse_poly_degree, its
    degree lowered by P_CoarsStgy (Minus1, Minus2 by default, DivideBy2, DirectToLow) and never below
    coarse_poly_degree (CoarsePolyDegree, 1 by default)."""
    if strategy not in P_STRATEGIES:
        raise ValueError(f"unknown p-coarsening strategy {strategy!r} ({', '.join(P_STRATEGIES)})")
    if k <= coarse_poly_degree:
        raise ValueError("p-coarsening cannot be performed because the polynomial degree of the fine level = "
                         f"{coarse_poly_degree}")
    degs = [k]
    while n_faces * face_unknowns(dim, degs[-1]) > max_coarse_rows and degs[-1] > coarse_poly_degree:
        d = degs[-1]
        c = {"minus1": d - 1, "minus2": d - 2, "divide_by_2": d // 2, "direct_to_low": coarse_poly_degree}[strategy]
        degs.append(max(c, coarse_poly_degree))
    return degs


def generate_p(dim: int, n: int, k: int, coarse_solver: str = "ch", strategy: str = "minus2",
               coarse_poly_degree: int = 1, max_coarse_rows: int = 1000, **kw):
    """The hierarchy of FCG with the p-multigrid preconditioner ("-s fcg -p p_mg", SolverFactory.h:201-211):
    the p-levels on the fine mesh (face degrees from p_degrees, joined by the natural injection),
    then, with the coarse solver "mg", the levels below the finest of the lowest degree's h-multigrid
    (the coarse solver SolverFactory.h:289-309 builds for "-cs mg": one cycle with no pre-smoothing
    and 3 (2D) or 6 (3D) post-smoothing steps). With "ch" (the default) the lowest degree is the
    coarsest level, solved directly.

    Returns (As, Ps, b, block_sizes, coarse_nu): coarse_nu is the pre and post smoothing of levels
    >= 1 that reproduces the reference's cycle ((-1, -1): those of level 0)."""
    if coarse_solver not in ("ch", "mg"):
        raise ValueError("coarse solver 'ch' (direct) or 'mg' (one h-multigrid cycle)")
    H = Hierarchy(dim, n, k, max_coarse_rows=max_coarse_rows, **kw)
    try:
        As, b, bss = [H.A(0)], H.b(), [H.block_size]
    finally:
        H.close()
    n_faces = As[0].shape[0] // bss[0]
    degs = p_degrees(dim, k, n_faces, strategy, coarse_poly_degree, max_coarse_rows)
    if coarse_solver == "mg" and len(degs) > 2:
        raise NotImplementedError("with the h-multigrid coarse solver the p-levels between the finest and the "
                                  "lowest degree would need smoothing counts of their own")
    if coarse_solver == "mg" and len(degs) == 1:
        raise NotImplementedError("the fine level is already the lowest-degree level: the h-multigrid coarse "
                                  "solver would smooth it with counts of its own")
    Ps = []
    for d in degs[1:]:
        nl = face_unknowns(dim, d)
        Ps.append(natural_injection(n_faces, bss[-1], nl))
        bss.append(nl)
        Hd = Hierarchy(dim, n, d, max_coarse_rows=max_coarse_rows, **kw)
        try:
            As.append(Hd.A(0))
            if d == degs[-1] and coarse_solver == "mg":
                for l in range(1, Hd.levels):
                    Ps.append(Hd.P(l - 1))
                    As.append(Hd.A(l))
                    bss.append(nl)
        finally:
            Hd.close()
    coarse_nu = (0, 3 if dim == 2 else 6) if coarse_solver == "mg" else (-1, -1)
    return As, Ps, b, bss, coarse_nu
