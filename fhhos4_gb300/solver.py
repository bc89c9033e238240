"""Python mirror of the reference's solver interface for the solve phase.

Names, attributes and defaults follow fhhos4's C++ classes so that code written
against them reads the same:

* ``IterativeSolver`` (src/Solver/IterativeSolver.h:6-191): ``Tolerance``,
  ``MaxIterations``, ``IterationCount``, ``OnIterationEnd``, ``Setup(A)``,
  ``Solve(b, initialGuessCode="0")``.
* ``Multigrid`` (src/Solver/Multigrid/Multigrid.h:7-46): cycle and smoother fields; its
  levels are the operators and prolongations that ``LevelForHHO`` builds
  (src/Solver/Multigrid/MultigridForHHO/LevelForHHO.h:72-213), given here with
  ``SetHierarchy``.
* ``SolverPreconditioner`` (src/Solver/Preconditioner.h:100-118): one V-cycle per
  application.
* ``FlexibleConjugateGradient(truncation=1)`` (src/Solver/Krylov/FlexibleConjugateGradient.h)
  and ``ConjugateGradient`` (src/Solver/Krylov/ConjugateGradient.h).

Everything runs in libfhg on the GPU; there is no CPU path. The reference reports
errors with ``Utils::FatalError`` (print + exit); here the same conditions raise
:class:`fhhos4_gb300._native.FhgError` with the reference's message.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, List, Optional

import numpy as np
import scipy.sparse as sp

from . import _native as N


# Smoother codes that SmootherFactory::Create (src/Solver/Multigrid/SmootherFactory.h:37-100) maps to
# the same smoother as a GPU code: the block SOR names are the Gauss-Seidel codes (block SOR when
# RelaxationParameter != 1, block GS when it is 1), and the hybrid chunk-parallel sweeps "hbgs" /
# "hrbgs" (BlockGaussSeidel.h:124-185, whose result depends on the host thread schedule) run as
# the multicolour parallel sweeps.
SMOOTHER_ALIASES = {"bsor": "bgs", "rbsor": "rbgs", "sbsor": "sbgs", "absor": "abgs", "rabsor": "rabgs",
                    "hbgs": "bgs", "hrbgs": "rbgs"}


def smoother_code(code: str) -> int:
    """libfhg's code of a reference smoother code; NotImplementedError for the others."""
    code = SMOOTHER_ALIASES.get(code, code)
    if code not in N.SMOOTHERS:
        raise NotImplementedError(f"smoother '{code}' (GPU smoothers: {sorted(N.SMOOTHERS) + sorted(SMOOTHER_ALIASES)})")
    return N.SMOOTHERS[code]


def as_eigen_csr(A) -> sp.csr_matrix:
    """Row-major CSR with int32 indices, sorted and duplicate-free (Eigen compressed form)."""
    A = sp.csr_matrix(A)
    A.sum_duplicates()
    A.sort_indices()
    return sp.csr_matrix((A.data.astype(np.float64), A.indices.astype(np.int32), A.indptr.astype(np.int32)),
                         shape=A.shape)


@dataclass
class IterationResult:
    """The fields of IterationResult (src/Solver/IterationResult.h:23-33) the solve phase fills."""
    IterationNumber: int = 0
    NormalizedResidualNorm: float = -1.0
    PreviousNormalizedResidualNorm: float = -1.0
    IterationConvRate: float = 0.0
    AsymptoticConvRate: float = 0.0


class IterativeSolver:
    def __init__(self):
        self.Tolerance = 1e-3
        self.MaxIterations = 200
        self.IterationCount = 0
        self.PrintIterationResults = False
        self.OnIterationEnd: Optional[Callable[[IterationResult], None]] = None
        self.LastIterationResult = IterationResult()
        self.Matrix = None
        self.SolveTimeMs = 0.0
        self.History = np.zeros(0)

    def Setup(self, A):
        self.Matrix = as_eigen_csr(A)


class Multigrid(IterativeSolver):
    """Geometric multigrid (V-cycle) over a given hierarchy, executed by libfhg."""

    def __init__(self, nLevels: int = 0):
        super().__init__()
        self.Cycle = "V"
        self.WLoops = 1
        self.PreSmootherCode = "bgs"
        self.PostSmootherCode = "rbgs"
        self.PreSmoothingIterations = 1
        self.PostSmoothingIterations = 1
        self.RelaxationParameter = 1.0
        self.BlockSizeForBlockSmoothers = -1
        self.MatrixMaxSizeForCoarsestLevel = 1000
        self.UseGalerkinOperator = False   # coarse operators P^T A P (Level.h:133-137, "-g 1")
        # GB300 knobs
        self.VCyclePrecision = "fp64"
        self.Colouring = True
        self.Autotune = False
        self.MaxCoarseRows = 8192
        # smoothing steps on levels >= 1; -1: PreSmoothingIterations / PostSmoothingIterations
        self.CoarsePreSmoothingIterations = -1
        self.CoarsePostSmoothingIterations = -1
        self.GsLayout = "auto"   # FP32 GS sweeps: "auto", "row" or "slot" (padded rows)
        # further V-cycle precisions whose operator copies setup builds, to switch to later
        self.ExtraPrecisions: List[str] = []
        self._As: List[sp.csr_matrix] = []
        self._Ps: List[sp.csr_matrix] = []
        self._BlockSizes: Optional[List[int]] = None
        self._nLevels = nLevels

    def SetHierarchy(self, As, Ps, block_sizes=None):
        """A_0..A_{L-1} and P_0..P_{L-2} (P_l: level l rows, level l+1 columns), as built on the host.
        block_sizes: one per level where they differ (a p-multigrid hierarchy, P_MultigridForHHO.h:
        levels of lower face degree joined by the natural injection); None: BlockSizeForBlockSmoothers
        on every level."""
        if len(Ps) != len(As) - 1:
            raise ValueError("need one prolongation per level except the coarsest")
        if block_sizes is not None and len(block_sizes) != len(As):
            raise ValueError("need one block size per level")
        self._As = [as_eigen_csr(A) for A in As]
        self._Ps = [as_eigen_csr(P) for P in Ps]
        self._BlockSizes = None if block_sizes is None else [int(b) for b in block_sizes]
        self._nLevels = len(As)

    def NumberOfLevels(self) -> int:
        return self._nLevels

    def _check_supported(self):
        if self.Cycle not in ("V", "W", "K"):
            raise NotImplementedError("V-, W- and K-cycles run on the GPU (Cycle='V', 'W' or 'K')")
        if self.Cycle == "W" and self.WLoops < 2:
            self.WLoops = 2
        for code in (self.PreSmootherCode, self.PostSmootherCode):
            smoother_code(code)
        if self.VCyclePrecision not in N.PRECISION:
            raise ValueError(f"unknown precision {self.VCyclePrecision}")


class SolverPreconditioner:
    """One application = one V-cycle from zero (Preconditioner.h:107-118,162-167)."""

    def __init__(self, solver: Optional[Multigrid] = None):
        self._solver = solver
        if solver is not None:
            solver.MaxIterations = 1


class _KrylovOnGpu(IterativeSolver):
    _krylov = "fcg"

    def __init__(self):
        super().__init__()
        self.Precond = SolverPreconditioner()
        self.Device = 0
        self.UseGraphs = True
        # FP32 V-cycle only: apply the outer operator in double-FP32 arithmetic (FP64-class
        # accuracy on the FP32 pipe) instead of native FP64.
        self.OuterSplit = True
        # Residual replacement in every precision (the FP32 V-cycle always replaces); off keeps the
        # reference's stopping loop in FP64.
        self.ReplaceResidual = False
        # the coarse part of the cycle as one cluster launch where the levels are small (FP32 / DF);
        # "wide": the same with 1024-thread CTAs when the launch shape is not timed
        self.FusedCoarse = True
        self._ctx: Optional[N.Context] = None

    def _options(self, mg: Multigrid) -> N.Options:
        o = N.default_options()
        o.krylov = N.KRYLOV[self._krylov]
        o.pre_smoother = smoother_code(mg.PreSmootherCode)
        o.post_smoother = smoother_code(mg.PostSmootherCode)
        o.pre_iterations = mg.PreSmoothingIterations
        o.post_iterations = mg.PostSmoothingIterations
        o.omega = mg.RelaxationParameter
        o.tolerance = self.Tolerance
        o.max_iterations = self.MaxIterations
        o.vcycle_precision = N.PRECISION[mg.VCyclePrecision]
        o.colouring = 1 if mg.Colouring else 0
        o.use_graphs = 1 if self.UseGraphs else 0
        o.autotune = 1 if mg.Autotune else 0
        o.max_coarse_rows = mg.MaxCoarseRows
        o.outer_split = 1 if self.OuterSplit else 0
        o.replace_residual = 1 if self.ReplaceResidual else 0
        o.fused_coarse = 2 if self.FusedCoarse == "wide" else (1 if self.FusedCoarse else 0)
        o.w_loops = N.CYCLE_K if mg.Cycle == "K" else (mg.WLoops if mg.Cycle == "W" else 1)
        o.galerkin = 1 if mg.UseGalerkinOperator else 0
        o.coarse_pre_iterations = mg.CoarsePreSmoothingIterations
        o.coarse_post_iterations = mg.CoarsePostSmoothingIterations
        o.gs_layout = N.GS_LAYOUT[mg.GsLayout]
        o.extra_precisions = sum(1 << N.PRECISION[p] for p in set(mg.ExtraPrecisions))
        return o

    def Setup(self, A):
        """FlexibleConjugateGradient::Setup (FlexibleConjugateGradient.h:32-37): the operator and the
        preconditioner's whole hierarchy go to the GPU."""
        super().Setup(A)
        mg = self.Precond._solver
        if mg is None:
            raise NotImplementedError("the GPU Krylov solvers need the multigrid preconditioner")
        mg._check_supported()
        if not mg._As:
            raise ValueError("Multigrid.SetHierarchy must be called before Setup")
        if mg._As[0].shape != self.Matrix.shape:
            raise ValueError("the finest multigrid level is not the system matrix")
        bs = mg.BlockSizeForBlockSmoothers
        if bs <= 0:
            raise ValueError("BlockSizeForBlockSmoothers must be set (face DOFs)")
        bss = mg._BlockSizes or [bs] * len(mg._As)
        if bss[0] != bs:
            raise ValueError("the finest level's block size is not BlockSizeForBlockSmoothers")
        if self._ctx is None:
            self._ctx = N.Context(self.Device)
        self._ctx.set_level(0, bs, self.Matrix)
        for l in range(1, len(mg._As)):
            self._ctx.set_level(l, bss[l], mg._As[l])
        for l, P in enumerate(mg._Ps):
            self._ctx.set_prolongation(l, P)
        self._ctx.setup(len(mg._As), self._options(mg))

    def Solve(self, b, initialGuessCode: str = "0"):
        """IterativeSolver::Solve(b, "0") (IterativeSolver.h:55-73)."""
        if initialGuessCode != "0":
            raise NotImplementedError("the GPU solve starts from x = 0 (initial guess code \"0\")")
        if self._ctx is None:
            raise N.FhgError(N.FHG_ERR_NOT_READY, "Setup has not been called")
        rc, x, hist, info = self._ctx.solve(np.asarray(b, dtype=np.float64), self.MaxIterations)
        self.IterationCount = info.iterations
        self.SolveTimeMs = info.solve_ms
        self.TrueRelativeResidual = info.true_relative_residual
        self.History = hist
        prev = -1.0
        rates: List[float] = []
        for k, nr in enumerate(hist):
            r = IterationResult(IterationNumber=k, NormalizedResidualNorm=float(nr), PreviousNormalizedResidualNorm=prev)
            if prev != -1.0:
                r.IterationConvRate = nr / prev
                rates = (rates + [r.IterationConvRate])[-5:]
                r.AsymptoticConvRate = float(np.prod(rates) ** (1.0 / len(rates)))
            if self.OnIterationEnd:
                self.OnIterationEnd(r)
            self.LastIterationResult = r
            prev = nr
        if rc != N.FHG_OK:
            self._ctx._check(rc)
        return x

    def Context(self) -> N.Context:
        return self._ctx


class FlexibleConjugateGradient(_KrylovOnGpu):
    _krylov = "fcg"

    def __init__(self, truncation: int = 1, restart: bool = False):
        super().__init__()
        if truncation != 1 or restart:
            raise NotImplementedError("FCG(1) without restart is the configuration on the GPU")
        self.Truncation = truncation
        self.Restart = restart


class ConjugateGradient(_KrylovOnGpu):
    _krylov = "cg"


def fcg_mg(As, Ps, block_size, tol: float = 1e-8, maxit: int = 200, pre: str = "bgs", post: str = "rbgs",
           precision: str = "fp64", krylov: str = "fcg", device: int = 0, autotune: bool = False,
           use_graphs: bool = True, outer_split: bool = True, cycle: str = "V", galerkin: bool = False,
           nu=(1, 1), coarse_nu=(-1, -1), gs_layout: str = "auto", omega: float = 1.0, extra=(),
           replace_residual: bool = False, fused: bool = True, colouring: bool = True):
    """SolverFactory-style construction of "-s fcgmg -cycle V,1,1" (src/Solver/SolverFactory.h:156-200).
    block_size: the face block size, or one per level (a p-multigrid hierarchy, hho.generate_p)."""
    mg = Multigrid(len(As))
    per_level = np.ndim(block_size) > 0
    mg.SetHierarchy(As, Ps, list(block_size) if per_level else None)
    mg.BlockSizeForBlockSmoothers = int(block_size[0]) if per_level else block_size
    mg.PreSmootherCode, mg.PostSmootherCode = pre, post
    mg.VCyclePrecision = precision
    mg.Autotune = autotune
    mg.Cycle = cycle
    mg.WLoops = 2 if cycle == "W" else 1
    mg.UseGalerkinOperator = galerkin
    mg.PreSmoothingIterations, mg.PostSmoothingIterations = nu
    mg.CoarsePreSmoothingIterations, mg.CoarsePostSmoothingIterations = coarse_nu
    mg.GsLayout = gs_layout
    mg.RelaxationParameter = omega
    mg.ExtraPrecisions = list(extra)
    mg.Colouring = colouring
    solver = FlexibleConjugateGradient(1) if krylov == "fcg" else ConjugateGradient()
    solver.Precond = SolverPreconditioner(mg)
    solver.Tolerance = tol
    solver.MaxIterations = maxit
    solver.Device = device
    solver.UseGraphs = use_graphs
    solver.OuterSplit = outer_split
    solver.ReplaceResidual = replace_residual
    solver.FusedCoarse = fused
    solver.Setup(As[0])
    return solver
