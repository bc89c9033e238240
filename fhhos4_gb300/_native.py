"""ctypes binding of libfhg.so (include/fhg.h).

The library is built in-tree by :mod:`fhhos4_gb300.build`; importing this module
never falls back to anything else: a missing library raises ``ImportError`` with
the build command, and every nonzero status raises :class:`FhgError`.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB

FHG_OK = 0
FHG_ERR_INVALID_ARG = -1
FHG_ERR_CUDA = -2
FHG_ERR_NOT_READY = -3
FHG_ERR_SINGULAR_BLOCK = -4
FHG_ERR_NOT_SPD = -5
FHG_ERR_DIVERGED = -6
FHG_ERR_NAN = -7
FHG_ERR_TOO_LARGE = -8
FHG_ERR_UNSUPPORTED = -9

SMOOTHERS = {"bgs": 0, "rbgs": 1, "bj": 2, "bj23": 3, "sbgs": 4, "abgs": 5, "rabgs": 6}
KRYLOV = {"fcg": 0, "cg": 1}
PRECISION = {"fp64": 0, "fp32": 1, "df": 2}   # df: FP64-class V-cycle in FP32 pairs (FHG_PREC_DF)

OP_SPMV, OP_RESIDUAL, OP_RESTRICT, OP_PROLONG_ADD = 0, 1, 2, 3
OP_GS_FORWARD, OP_GS_BACKWARD, OP_JACOBI, OP_SYM_SPMV = 4, 5, 6, 7
OP_COARSE_SOLVE, OP_VCYCLE, OP_VCYCLE_LEARNED, OP_LEARNED_STEP = 8, 9, 10, 11
CYCLE_K = -1   # fhg_options.w_loops / set_cycle: the K-cycle
GS_LAYOUT = {"auto": 0, "row": 1, "slot": 2}   # fhg_options.gs_layout
LEARNED = {"off": 0, "fallback": 1, "always": 2}
LEARNED_MMA_SYNC = 16
LEARNED_PARAMS = 24848

# Every symbol include/fhg.h declares.
EXPORTS = ["fhg_default_options", "fhg_create", "fhg_destroy", "fhg_last_error", "fhg_set_level",
           "fhg_set_prolongation", "fhg_setup", "fhg_solve", "fhg_solve_device", "fhg_apply",
           "fhg_time_op", "fhg_set_cycle", "fhg_set_coarse_smoothing", "fhg_set_vcycle_precision", "fhg_level_info", "fhg_fused_coarse_info", "fhg_device_bytes", "fhg_get_permutation",
           "fhg_kernel_launches", "fhg_residual_norm_noalloc", "fhg_set_face_tensors", "fhg_set_learned",
           "fhg_learned_reference_rate", "fhg_learned_features", "fhg_apply_internal", "fhg_net_num_params",
           "fhg_net_create", "fhg_net_destroy", "fhg_net_last_error", "fhg_net_set_params", "fhg_net_get_params",
           "fhg_net_train_step", "fhg_io_buffers", "fhg_io_upload", "fhg_io_download", "fhg_batch_create", "fhg_batch_destroy", "fhg_batch_last_error",
           "fhg_batch_add", "fhg_batch_solve", "fhg_post_create", "fhg_post_run", "fhg_post_last_error",
           "fhg_post_destroy", "fhg_cond_create", "fhg_cond_run", "fhg_cond_result", "fhg_cond_download", "fhg_cond_last_error",
           "fhg_cond_destroy"]

FHG_NOALLOC_MAX_PARTIALS = 131072


class FhgError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"fhg error {code}: {message}")
        self.code = code


class Options(C.Structure):
    _fields_ = [("krylov", C.c_int), ("pre_smoother", C.c_int), ("post_smoother", C.c_int),
                ("pre_iterations", C.c_int), ("post_iterations", C.c_int), ("omega", C.c_double),
                ("tolerance", C.c_double), ("max_iterations", C.c_int), ("vcycle_precision", C.c_int),
                ("colouring", C.c_int), ("use_graphs", C.c_int), ("autotune", C.c_int),
                ("max_coarse_rows", C.c_int), ("outer_split", C.c_int), ("w_loops", C.c_int),
                ("galerkin", C.c_int), ("coarse_pre_iterations", C.c_int), ("coarse_post_iterations", C.c_int),
                ("gs_layout", C.c_int), ("extra_precisions", C.c_int), ("replace_residual", C.c_int),
                ("fused_coarse", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("status", C.c_int), ("normalized_residual", C.c_double),
                ("solve_ms", C.c_double), ("learned_iterations", C.c_int), ("true_relative_residual", C.c_double)]


_lib = None


def load(path: str = LIB):
    """Load libfhg.so (raises ImportError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m fhhos4_gb300.build`")
    lib = C.CDLL(path)
    P = C.POINTER
    lib.fhg_default_options.argtypes = [P(Options)]
    lib.fhg_default_options.restype = None
    lib.fhg_create.argtypes = [P(C.c_void_p), C.c_int]
    lib.fhg_destroy.argtypes = [C.c_void_p]
    lib.fhg_destroy.restype = None
    lib.fhg_last_error.argtypes = [C.c_void_p]
    lib.fhg_last_error.restype = C.c_char_p
    lib.fhg_set_level.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.fhg_set_prolongation.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.fhg_setup.argtypes = [C.c_void_p, C.c_int, P(Options)]
    lib.fhg_solve.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, P(SolveInfo)]
    lib.fhg_solve_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, P(SolveInfo)]
    lib.fhg_apply.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.fhg_time_op.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, P(C.c_double)]
    lib.fhg_set_vcycle_precision.argtypes = [C.c_void_p, C.c_int]
    lib.fhg_set_cycle.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
    lib.fhg_set_coarse_smoothing.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.fhg_fused_coarse_info.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_int), P(C.c_int)]
    lib.fhg_device_bytes.argtypes = [C.c_void_p]
    lib.fhg_device_bytes.restype = C.c_longlong
    lib.fhg_level_info.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(C.c_longlong), P(C.c_int), P(C.c_int),
                                   P(C.c_longlong)]
    lib.fhg_get_permutation.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    lib.fhg_kernel_launches.argtypes = [C.c_void_p]
    lib.fhg_kernel_launches.restype = C.c_longlong
    lib.fhg_residual_norm_noalloc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.fhg_set_face_tensors.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    lib.fhg_set_learned.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    lib.fhg_learned_reference_rate.argtypes = [C.c_void_p, P(C.c_double)]
    lib.fhg_learned_features.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.fhg_apply_internal.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.fhg_net_num_params.argtypes = []
    lib.fhg_net_create.argtypes = [P(C.c_void_p), C.c_int]
    lib.fhg_net_destroy.argtypes = [C.c_void_p]
    lib.fhg_net_destroy.restype = None
    lib.fhg_net_last_error.argtypes = [C.c_void_p]
    lib.fhg_net_last_error.restype = C.c_char_p
    lib.fhg_net_set_params.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    lib.fhg_net_get_params.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    lib.fhg_net_train_step.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_float, C.c_float, C.c_int,
                                       P(C.c_double), C.c_void_p]
    lib.fhg_io_buffers.argtypes = [C.c_void_p, P(C.c_void_p), P(C.c_void_p)]
    lib.fhg_io_upload.argtypes = [C.c_void_p, C.c_void_p]
    lib.fhg_io_download.argtypes = [C.c_void_p, C.c_void_p]
    lib.fhg_batch_create.argtypes = [P(C.c_void_p), C.c_int]
    lib.fhg_batch_destroy.argtypes = [C.c_void_p]
    lib.fhg_batch_destroy.restype = None
    lib.fhg_batch_last_error.argtypes = [C.c_void_p]
    lib.fhg_batch_last_error.restype = C.c_char_p
    lib.fhg_batch_add.argtypes = [C.c_void_p, C.c_void_p]
    lib.fhg_batch_solve.argtypes = [C.c_void_p, C.c_void_p, P(C.c_double)]
    lib.fhg_post_create.argtypes = [P(C.c_void_p)] + [C.c_int] * 8 + [C.c_void_p] * 9
    lib.fhg_post_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, P(C.c_double), P(C.c_double)]
    lib.fhg_post_last_error.argtypes = [C.c_void_p]
    lib.fhg_post_last_error.restype = C.c_char_p
    lib.fhg_post_destroy.argtypes = [C.c_void_p]
    lib.fhg_post_destroy.restype = None
    lib.fhg_cond_create.argtypes = [P(C.c_void_p)] + [C.c_int] * 7 + [C.c_void_p] * 5
    lib.fhg_cond_run.argtypes = [C.c_void_p, P(C.c_longlong), P(C.c_double)]
    lib.fhg_cond_result.argtypes = [C.c_void_p, P(C.c_void_p), P(C.c_void_p), P(C.c_void_p), P(C.c_void_p)]
    lib.fhg_cond_download.argtypes = [C.c_void_p] + [C.c_void_p] * 4
    lib.fhg_cond_last_error.argtypes = [C.c_void_p]
    lib.fhg_cond_last_error.restype = C.c_char_p
    lib.fhg_cond_destroy.argtypes = [C.c_void_p]
    lib.fhg_cond_destroy.restype = None
    _lib = lib
    return lib


def ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data) if a is not None else None


class Context:
    """Owns one fhg_ctx (one hierarchy on one GPU)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.h = C.c_void_p()
        rc = self.lib.fhg_create(C.byref(self.h), device)
        self._check(rc)

    def _check(self, rc: int):
        if rc != FHG_OK:
            msg = self.lib.fhg_last_error(self.h).decode() if self.h else "no context"
            raise FhgError(rc, msg)

    def close(self):
        if self.h:
            self.lib.fhg_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- hierarchy -------------------------------------------------------
    def set_level(self, level: int, block_size: int, A):
        rp = np.ascontiguousarray(A.indptr, dtype=np.int32)
        ci = np.ascontiguousarray(A.indices, dtype=np.int32)
        va = np.ascontiguousarray(A.data, dtype=np.float64)
        self._check(self.lib.fhg_set_level(self.h, level, block_size, A.shape[0], ptr(rp), ptr(ci), ptr(va)))

    def set_prolongation(self, level: int, P):
        rp = np.ascontiguousarray(P.indptr, dtype=np.int32)
        ci = np.ascontiguousarray(P.indices, dtype=np.int32)
        va = np.ascontiguousarray(P.data, dtype=np.float64)
        self._check(self.lib.fhg_set_prolongation(self.h, level, P.shape[0], P.shape[1], ptr(rp), ptr(ci), ptr(va)))

    def setup(self, nlevels: int, opts: Options):
        self._check(self.lib.fhg_setup(self.h, nlevels, C.byref(opts)))

    # -- solve -----------------------------------------------------------
    def solve(self, b: np.ndarray, max_iterations: int):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.empty_like(b)
        hist = np.zeros(max_iterations + 1)
        info = SolveInfo()
        rc = self.lib.fhg_solve(self.h, ptr(b), ptr(x), ptr(hist), C.byref(info))
        return rc, x, hist[: info.iterations + 1].copy(), info

    def solve_device(self, b_dev_ptr: int, x_dev_ptr: int, max_iterations: int):
        hist = np.zeros(max_iterations + 1)
        info = SolveInfo()
        rc = self.lib.fhg_solve_device(self.h, C.c_void_p(b_dev_ptr), C.c_void_p(x_dev_ptr), ptr(hist),
                                       C.byref(info))
        return rc, hist[: info.iterations + 1].copy(), info

    def apply(self, level: int, op: int, inp: np.ndarray, aux: np.ndarray | None, n_out: int):
        inp = np.ascontiguousarray(inp, dtype=np.float64)
        auxa = None if aux is None else np.ascontiguousarray(aux, dtype=np.float64)
        out = np.empty(n_out)
        self._check(self.lib.fhg_apply(self.h, level, op, ptr(inp), ptr(auxa), ptr(out)))
        return out

    def time_op(self, level: int, op: int, precision: str = "fp64", warmup: int = 3, reps: int = 20) -> float:
        ms = C.c_double()
        self._check(self.lib.fhg_time_op(self.h, level, op, PRECISION[precision], warmup, reps, C.byref(ms)))
        return ms.value

    def set_cycle(self, pre: str = "bgs", post: str = "rbgs", npre: int = 1, npost: int = 1, w_loops: int = 1):
        self._check(self.lib.fhg_set_cycle(self.h, SMOOTHERS[pre], SMOOTHERS[post], npre, npost, w_loops))

    def set_coarse_smoothing(self, npre: int = -1, npost: int = -1):
        """Smoothing steps on levels >= 1 (-1: those of level 0)."""
        self._check(self.lib.fhg_set_coarse_smoothing(self.h, npre, npost))

    def set_vcycle_precision(self, precision: str):
        self._check(self.lib.fhg_set_vcycle_precision(self.h, PRECISION[precision]))

    def level_info(self, level: int):
        nb, nbl, nc, lanes, pb = C.c_int(), C.c_longlong(), C.c_int(), C.c_int(), C.c_longlong()
        self._check(self.lib.fhg_level_info(self.h, level, C.byref(nb), C.byref(nbl), C.byref(nc), C.byref(lanes),
                                            C.byref(pb)))
        return dict(block_rows=nb.value, blocks=nbl.value, colours=nc.value, lanes=lanes.value, p_blocks=pb.value)

    def device_bytes(self) -> int:
        """Device memory the context holds, in bytes."""
        return int(self.lib.fhg_device_bytes(self.h))

    def fused_coarse_info(self, precision: str):
        """(first level of the one-launch coarse sub-cycle or -1, CTAs of its cluster, threads of a
        CTA) as run now."""
        first, ctas, threads = C.c_int(), C.c_int(), C.c_int()
        self._check(self.lib.fhg_fused_coarse_info(self.h, PRECISION[precision], C.byref(first), C.byref(ctas),
                                                   C.byref(threads)))
        return first.value, ctas.value, threads.value

    def permutation(self, level: int, nb: int) -> np.ndarray:
        perm = np.empty(nb, dtype=np.int32)
        self._check(self.lib.fhg_get_permutation(self.h, level, ptr(perm)))
        return perm

    def kernel_launches(self) -> int:
        return int(self.lib.fhg_kernel_launches(self.h))

    # -- learned correction ----------------------------------------------
    def set_face_tensors(self, tensors: np.ndarray):
        t = np.ascontiguousarray(tensors, dtype=np.float64)
        if t.ndim != 2 or t.shape[1] != 12:
            raise ValueError("face tensors are (n_blocks, 12)")
        self._check(self.lib.fhg_set_face_tensors(self.h, t.shape[0], ptr(t)))

    def set_learned(self, params: np.ndarray | None, mode: str = "fallback", kernel: str = "tcgen05"):
        """Install a network (None keeps the installed one) and select the mode; kernel "tcgen05"
        (tensor-memory accumulators) or "mma_sync"."""
        m = LEARNED[mode] | (LEARNED_MMA_SYNC if kernel == "mma_sync" else 0)
        if params is None:
            self._check(self.lib.fhg_set_learned(self.h, None, 0, m))
            return
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(self.lib.fhg_set_learned(self.h, ptr(p), p.size, m))

    def learned_reference_rate(self) -> float:
        r = C.c_double()
        self._check(self.lib.fhg_learned_reference_rate(self.h, C.byref(r)))
        return r.value

    def learned_features(self, r_dev: int, features_dev: int, scale_dev: int):
        self._check(self.lib.fhg_learned_features(self.h, C.c_void_p(r_dev), C.c_void_p(features_dev),
                                                  C.c_void_p(scale_dev)))

    def apply_internal(self, level: int, op: int, precision: str, in_dev: int, aux_dev: int | None, out_dev: int):
        """One operator on device vectors in the context's colour numbering (see fhg_apply_internal)."""
        self._check(self.lib.fhg_apply_internal(self.h, level, op, PRECISION[precision], C.c_void_p(in_dev),
                                                C.c_void_p(aux_dev) if aux_dev else None, C.c_void_p(out_dev)))


    def io_buffers(self):
        """(b_dev, x_dev): the context's device vectors read and written by a batched solve."""
        b, x = C.c_void_p(), C.c_void_p()
        self._check(self.lib.fhg_io_buffers(self.h, C.byref(b), C.byref(x)))
        return b.value, x.value

    def io_upload(self, b: np.ndarray):
        b = np.ascontiguousarray(b, dtype=np.float64)
        self._check(self.lib.fhg_io_upload(self.h, ptr(b)))

    def io_download(self, n: int) -> np.ndarray:
        x = np.empty(n)
        self._check(self.lib.fhg_io_download(self.h, ptr(x)))
        return x


class Batch:
    """Owns one fhg_batch: set-up contexts solved together by one graph launch."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.h = C.c_void_p()
        self._ctxs = []
        self._check(self.lib.fhg_batch_create(C.byref(self.h), device))

    def _check(self, rc: int):
        if rc != FHG_OK:
            msg = self.lib.fhg_batch_last_error(self.h).decode() if self.h else "no batch"
            raise FhgError(rc, msg)

    def add(self, ctx: "Context"):
        self._check(self.lib.fhg_batch_add(self.h, ctx.h))
        self._ctxs.append(ctx)

    def solve(self):
        """Returns (status, [SolveInfo per context], elapsed ms of the launch)."""
        infos = (SolveInfo * len(self._ctxs))()
        ms = C.c_double()
        rc = self.lib.fhg_batch_solve(self.h, infos, C.byref(ms))
        return rc, list(infos), ms.value

    def close(self):
        if self.h:
            self.lib.fhg_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


EXACT = {"none": 0, "sine": 1}


class Post:
    """Owns one fhg_post: the finest level's element tables on a GPU, for cell-unknown recovery and
    the L2 error of the k+1 reconstruction (tables as fhhos4_gb300.hho.Hierarchy.post_tables gives)."""

    def __init__(self, tables: dict, device: int = 0):
        self.lib = load()
        self.h = C.c_void_p()
        t = {k: np.ascontiguousarray(v) for k, v in tables.items() if isinstance(v, np.ndarray)}
        self._keep = t
        self.n_elements, self.n_cell = int(tables["n_elements"]), int(tables["n_cell"])
        self._check(self.lib.fhg_post_create(
            C.byref(self.h), device, int(tables["dim"]), self.n_elements, int(tables["n_classes"]), self.n_cell,
            int(tables["n_face_dofs"]), int(tables["n_recon"]), int(tables["n_points"]),
            ptr(t["elem_class"]), ptr(t["elem_faces"]), ptr(t["elem_centre"]), ptr(t["cell_rhs"]),
            ptr(t["solve_cells"]), ptr(t["recon"]), ptr(t["weights"]), ptr(t["offsets"]), ptr(t["basis"])))

    def _check(self, rc: int):
        if rc != FHG_OK:
            msg = self.lib.fhg_post_last_error(self.h).decode() if self.h else "no post-processing handle"
            raise FhgError(rc, msg)

    def run(self, x_faces_dev: int, x_cells_dev: int = 0, exact: str = "sine"):
        """(relative L2 error or None, device ms) for the face solution at device address x_faces_dev;
        cell unknowns written to x_cells_dev (n_elements x n_cell doubles) when given."""
        err, ms = C.c_double(), C.c_double()
        self._check(self.lib.fhg_post_run(self.h, C.c_void_p(x_faces_dev), C.c_void_p(x_cells_dev) if x_cells_dev else None,
                                          EXACT[exact], C.byref(err), C.byref(ms)))
        return (err.value if exact != "none" else None), ms.value

    def close(self):
        if self.h:
            self.lib.fhg_post_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Condense:
    """Owns one fhg_cond: static condensation and assembly of the finest face system on a GPU
    (tables as fhhos4_gb300.hho.Hierarchy.condense_tables gives)."""

    def __init__(self, tables: dict, device: int = 0):
        self.lib = load()
        self.h = C.c_void_p()
        t = {k: np.ascontiguousarray(v) for k, v in tables.items() if isinstance(v, np.ndarray)}
        self._keep = t
        self.nf = int(tables["n_face_dofs"]) // (int(tables["dim"]) + 1)
        self.n_face_blocks = int(tables["n_face_blocks"])
        self._check(self.lib.fhg_cond_create(
            C.byref(self.h), device, int(tables["dim"]), int(tables["n_elements"]), int(tables["n_classes"]),
            int(tables["n_cell"]), int(tables["n_face_dofs"]), self.n_face_blocks, ptr(t["elem_class"]),
            ptr(t["elem_faces"]), ptr(t["face_elems"]), ptr(t["local"]), ptr(t["b_cell"])))

    def _check(self, rc: int):
        if rc != FHG_OK:
            msg = self.lib.fhg_cond_last_error(self.h).decode() if self.h else "no condensation handle"
            raise FhgError(rc, msg)

    def run(self):
        """Condense and assemble on the device: (stored entries, device ms)."""
        nnz, ms = C.c_longlong(), C.c_double()
        self._check(self.lib.fhg_cond_run(self.h, C.byref(nnz), C.byref(ms)))
        return nnz.value, ms.value

    def result(self, nnz: int):
        """The assembled system copied to the host: (scipy CSR A, b)."""
        import scipy.sparse as sp
        n = self.n_face_blocks * self.nf
        rowptr, colidx = np.empty(n + 1, np.int32), np.empty(nnz, np.int32)
        vals, b = np.empty(nnz), np.empty(n)
        self._check(self.lib.fhg_cond_download(self.h, ptr(rowptr), ptr(colidx), ptr(vals), ptr(b)))
        return sp.csr_matrix((vals, colidx, rowptr), shape=(n, n)), b

    def close(self):
        if self.h:
            self.lib.fhg_cond_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Net:
    """Owns one fhg_net: the network's FP32 parameters, Adam state and training buffers on a GPU."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self.h = C.c_void_p()
        rc = self.lib.fhg_net_create(C.byref(self.h), device)
        self._check(rc)
        self.n_params = int(self.lib.fhg_net_num_params())

    def _check(self, rc: int):
        if rc != FHG_OK:
            msg = self.lib.fhg_net_last_error(self.h).decode() if self.h else "no network"
            raise FhgError(rc, msg)

    def close(self):
        if self.h:
            self.lib.fhg_net_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params: np.ndarray):
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._check(self.lib.fhg_net_set_params(self.h, ptr(p), p.size))

    def params(self) -> np.ndarray:
        p = np.empty(self.n_params, dtype=np.float32)
        self._check(self.lib.fhg_net_get_params(self.h, ptr(p), p.size))
        return p

    def train_step(self, ctx: Context, r_dev: int, energy: float, lr: float, weight_decay: float = 0.0,
                   update: bool = True, want_grad: bool = False):
        """One step on one field; returns (loss before the update, gradient or None)."""
        loss = C.c_double()
        g = np.empty(self.n_params, dtype=np.float32) if want_grad else None
        self._check(self.lib.fhg_net_train_step(self.h, ctx.h, C.c_void_p(r_dev), float(energy), float(lr),
                                                float(weight_decay), 1 if update else 0, C.byref(loss), ptr(g)))
        return loss.value, g


def default_options() -> Options:
    o = Options()
    load().fhg_default_options(C.byref(o))
    return o
