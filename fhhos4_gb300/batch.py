"""Batched solve of many independent problems of uneven size (one graph launch, fhg_batch_*).

The workload generator follows the batched configuration: 2D unit squares, n x n cells split into
two triangles each, HHO degree k in {1, 2, 3} (face blocks of 2, 3, 4 unknowns), an isotropic
coefficient constant on each of 8 x 8 patches and log-uniform in [1e-3, 1e3], and a smooth source
made of four random sine modes with N(0, 1) amplitudes, all drawn from one seed.

n is drawn from the multiples of 16 in [32, 256]: the reference's geometric coarsening halves n
while it is even, so an n with a large odd factor leaves a coarsest level far above what a dense
direct solve takes (an odd n is a single level, i.e. a direct solve of the whole system). The
coarse operators are Galerkin products (Multigrid::UseGalerkinOperator, "-g 1"): with
rediscretised coarse operators the V-cycle is not a contraction when coarse cells straddle the
coefficient patches (n = 48, 80, 112, ...), and FCG does not converge.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import time
from dataclasses import dataclass
from typing import List

import numpy as np

from . import _native as N
from . import hho


@dataclass
class ProblemSpec:
    n: int
    k: int
    seed: int


def batched_specs(count: int, seed: int = 20261203, n_min: int = 32, n_max: int = 256, step: int = 16,
                  ks=(1, 2, 3)) -> List[ProblemSpec]:
    rng = np.random.default_rng(seed)
    ns = np.arange(n_min, n_max + 1, step)
    return [ProblemSpec(int(rng.choice(ns)), int(rng.choice(ks)), int(rng.integers(1, 2 ** 62))) for _ in range(count)]


def generate(spec: ProblemSpec, threads: int = 0):
    """The host hierarchy of one problem: (block size, A_0, [P_l], b, levels)."""
    H = hho.Hierarchy(2, spec.n, spec.k, source="modes", coefficient="lognormal_patches", contrast=1e3,
                      checker_blocks=8, seed=spec.seed, max_coarse_rows=1000, threads=threads)
    try:
        return H.block_size, H.A(0), [H.P(l) for l in range(H.levels - 1)], H.b(), H.levels
    finally:
        H.close()


class Problem:
    """One problem: its hierarchy on a set-up context; b uploaded to the context's device buffer."""

    def __init__(self, spec: ProblemSpec, device: int = 0, precision: str = "fp64", autotune: bool = True,
                 tol: float = 1e-8, maxit: int = 200, keep_operator: bool = False, generated=None, extra=()):
        bs, A0, Ps, b, levels = generated if generated is not None else generate(spec)
        self.spec = spec
        self.bs = bs
        self.b = b
        self.n = A0.shape[0]
        self.levels = levels
        ctx = N.Context(device)
        ctx.set_level(0, self.bs, A0)
        for l, P in enumerate(Ps):
            ctx.set_prolongation(l, P)
        o = N.default_options()
        o.galerkin = 1
        o.replace_residual = 1   # every precision: the FP64 true residual must meet the tolerance
        o.vcycle_precision = N.PRECISION[precision]
        o.extra_precisions = sum(1 << N.PRECISION[p] for p in set(extra))
        o.autotune = 1 if autotune else 0
        o.tolerance = tol
        o.max_iterations = maxit
        ctx.setup(self.levels, o)
        self.ctx = ctx
        self.A0 = A0 if keep_operator else None

    def upload_b(self):
        self.ctx.io_upload(self.b)

    def x(self) -> np.ndarray:
        return self.ctx.io_download(self.n)

    def close(self):
        if self.ctx is not None:
            self.ctx.close()
            self.ctx = None


def generate_all(specs: List[ProblemSpec]):
    """The host hierarchies of all problems, in parallel (one generator thread each; ctypes releases
    the GIL)."""
    workers = max(1, min(len(specs), os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(workers) as ex:
        return list(ex.map(lambda sp: generate(sp, threads=1), specs))


def build(specs: List[ProblemSpec], device: int = 0, precision: str = "fp64", autotune: bool = True,
          keep_operator: bool = False, extra=(), generated=None, threads: int = 0):
    """Problems with b uploaded, and a Batch holding all of them. Returns (problems, batch, seconds).
    generated: the hierarchies of generate_all(specs), reused; otherwise generated here. The contexts
    are set up on `threads` host threads (default: up to 16; ctypes releases the GIL, the library
    times one context at a time); on a failure every context made so far is closed and it re-raises."""
    t0 = time.time()
    gen = generated if generated is not None else generate_all(specs)
    workers = max(1, min(len(specs), threads or min(16, os.cpu_count() or 1)))
    with cf.ThreadPoolExecutor(workers) as ex:
        futs = [ex.submit(Problem, s, device, precision, autotune, keep_operator=keep_operator, generated=g, extra=extra)
                for s, g in zip(specs, gen)]
    probs, err = [], None
    for f in futs:
        try:
            probs.append(f.result())
        except Exception as e:  # noqa: BLE001 - closed below, then re-raised
            err = err or e
    if err is not None:
        for p in probs:
            p.close()
        raise err
    for p in probs:
        p.upload_b()
    batch = N.Batch(device)
    for p in probs:
        batch.add(p.ctx)
    return probs, batch, time.time() - t0
