"""Learned correction step of the FP32 V-cycle: training data, training on the GPU, evaluation.

The network (48-128-128-16, GELU, BF16 tensor cores with FP32 accumulation) and its kernels live
in libfhg (csrc/fhg_learned.cu); this module drives them:

* ``Field``: one seeded coefficient field on an in-house tetrahedral cube mesh, its hierarchy on a
  GPU context with the FP32 V-cycle, and the element tensors of every face.
* ``make_samples``: (residual, energy) pairs of errors left by the plain V-cycle: a seeded random
  error e0, then ``cycles`` plain V-cycles e <- e - V(A e), then r = A e, E = e.A e.
* ``train``: streams fields, takes Adam steps on the energy loss |e - c|_A^2 / |e|_A^2 of the
  network's correction c (fhg_net_train_step), cosine learning-rate decay.
* ``energy_ratio``: the same loss evaluated through the V-cycle itself, with and without the step.

Everything runs on the GPU through libfhg; torch only holds device vectors.
"""
from __future__ import annotations

import json
import math
import os
import time
from dataclasses import dataclass, field as dfield
from typing import List, Optional

import numpy as np

from . import _native as N
from . import hho

WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights")
DEFAULT_WEIGHTS = os.path.join(WEIGHTS_DIR, "learned_tet3d_k1.npz")

K_IN, K_HID, K_OUT = 48, 128, 16
OFF_W1 = 0
OFF_B1 = OFF_W1 + K_HID * K_IN
OFF_W2 = OFF_B1 + K_HID
OFF_B2 = OFF_W2 + K_HID * K_HID
OFF_W3 = OFF_B2 + K_HID
OFF_B3 = OFF_W3 + K_OUT * K_HID
N_PARAMS = OFF_B3 + K_OUT
assert N_PARAMS == N.LEARNED_PARAMS


def init_params(seed: int = 0, used_inputs: int = 33) -> np.ndarray:
    """Scaled-normal hidden layers (variance 1/fan-in), zero output layer: the untrained step adds
    nothing, so training starts from the plain V-cycle."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_PARAMS, dtype=np.float32)
    p[OFF_W1:OFF_B1] = (rng.standard_normal(K_HID * K_IN) / math.sqrt(used_inputs)).astype(np.float32)
    p[OFF_W2:OFF_B2] = (rng.standard_normal(K_HID * K_HID) / math.sqrt(K_HID)).astype(np.float32)
    return p


def save_params(path: str, params: np.ndarray, meta: dict):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez(path, params=np.asarray(params, dtype=np.float32), meta=json.dumps(meta))


def load_params(path: str = DEFAULT_WEIGHTS):
    with np.load(path) as z:
        return z["params"].astype(np.float32), json.loads(str(z["meta"]))


@dataclass
class FieldSpec:
    n: int = 16
    k: int = 1
    coefficient: str = "anisotropic"   # diag(1, 1, eps) rotated, eps log-uniform per 4^3 block
    eps_min: float = 1e-3
    contrast: float = 1.0
    checker_blocks: int = 0            # 0: one block per 4^3 cubes (n / 4 blocks per direction)
    seed: int = 1
    max_coarse_rows: int = 1000


def generate_field(spec: FieldSpec, source: str = "sine", threads: int = 0):
    """The host hierarchy of a field: (block size, [A_l], [P_l], b, face tensors of level 0)."""
    blocks = spec.checker_blocks or max(1, spec.n // 4)
    H = hho.Hierarchy(3, spec.n, spec.k, max_coarse_rows=spec.max_coarse_rows, source=source,
                      coefficient=spec.coefficient, contrast=spec.contrast, checker_blocks=blocks,
                      eps_min=spec.eps_min, seed=spec.seed, threads=threads)
    try:
        return (H.block_size, [H.A(l) for l in range(H.levels)], [H.P(l) for l in range(H.levels - 1)], H.b(),
                H.face_tensors(0))
    finally:
        H.close()


class Field:
    """One coefficient field: hierarchy on a GPU context (FP32 V-cycle) plus its face tensors."""

    def __init__(self, spec: FieldSpec, device: int = 0, smoothers=("bgs", "rbgs"), nu=(1, 1), autotune=False,
                 source: str = "sine", coarse_nu=(-1, -1), generated=None):
        self.spec = spec
        self.bs, self.As, Ps, self.b, self.tensors = generated if generated is not None else generate_field(spec, source)
        self.hierarchy = None
        self.n = self.As[0].shape[0]
        self.nb = self.n // self.bs
        ctx = N.Context(device)
        for l, A in enumerate(self.As):
            ctx.set_level(l, self.bs, A)
        for l, P in enumerate(Ps):
            ctx.set_prolongation(l, P)
        ctx.set_face_tensors(self.tensors)
        o = N.default_options()
        o.vcycle_precision = N.PRECISION["fp32"]
        o.pre_smoother, o.post_smoother = N.SMOOTHERS[smoothers[0]], N.SMOOTHERS[smoothers[1]]
        o.pre_iterations, o.post_iterations = nu
        o.coarse_pre_iterations, o.coarse_post_iterations = coarse_nu
        o.autotune = 1 if autotune else 0
        ctx.setup(len(self.As), o)
        self.ctx = ctx
        self.perm = ctx.permutation(0, self.nb)
        self.device = device

    def close(self):
        if self.ctx is not None:
            self.ctx.close()
            self.ctx = None
        if self.hierarchy is not None:
            self.hierarchy.close()
            self.hierarchy = None

    # device ops in the context's colour numbering (torch float32 vectors)
    def spmv(self, x, out):
        self.ctx.apply_internal(0, N.OP_SPMV, "fp32", x.data_ptr(), None, out.data_ptr())

    def vcycle(self, b, out, learned: bool = False):
        self.ctx.apply_internal(0, N.OP_VCYCLE_LEARNED if learned else N.OP_VCYCLE, "fp32", b.data_ptr(), None,
                                out.data_ptr())


def make_samples(f: Field, count: int, cycles=(1, 2, 3), seed: int = 0):
    """[(r, E)] with r = A e (device FP32, colour numbering) for errors e left by plain V-cycles."""
    import torch
    dev = torch.device("cuda", f.device)
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    out = []
    tmp = torch.empty(f.n, device=dev, dtype=torch.float32)
    z = torch.empty_like(tmp)
    for i in range(count):
        e = torch.randn(f.n, device=dev, dtype=torch.float32, generator=g)
        ncyc = cycles[i % len(cycles)]
        for _ in range(ncyc):
            torch.cuda.synchronize(dev)
            f.spmv(e, tmp)
            f.vcycle(tmp, z)
            e = e - z
            e = e / torch.linalg.vector_norm(e)
        r = torch.empty_like(e)
        torch.cuda.synchronize(dev)
        f.spmv(e, r)
        E = float(torch.dot(e.double(), r.double()))
        out.append((r, E, e))
    torch.cuda.synchronize(dev)
    return out


def energy_ratio(f: Field, e, learned: bool) -> float:
    """|e1|_A^2 / |e|_A^2 for one V-cycle applied to the residual of error e (plain or learned)."""
    import torch
    r = torch.empty_like(e)
    z = torch.empty_like(e)
    torch.cuda.synchronize()
    f.spmv(e, r)
    f.vcycle(r, z, learned=learned)
    e1 = e - z
    r1 = torch.empty_like(e)
    torch.cuda.synchronize()
    f.spmv(e1, r1)
    return float(torch.dot(e1.double(), r1.double()) / torch.dot(e.double(), r.double()))


@dataclass
class TrainLog:
    steps: int = 0
    fields: int = 0
    seconds: float = 0.0
    losses: List[float] = dfield(default_factory=list)


def train(net: N.Net, fields: int = 64, n: int = 16, samples_per_field: int = 4, steps_per_sample: int = 1,
          lr: float = 2e-3, lr_min: float = 1e-4, weight_decay: float = 0.0, seed0: int = 1000, device: int = 0,
          spec_kw: Optional[dict] = None, log_every: int = 0, smoothers=("bgs", "rbgs"), nu=(1, 1),
          identity_every: int = 0, coarse_nu=(-1, -1), sizes=None, prefetch: int = 0) -> TrainLog:
    """Stream `fields` seeded fields (seeds seed0, seed0+1, ...) and take Adam steps on their samples;
    identity_every = m > 0 makes every m-th field the identity coefficient instead. sizes: a list of
    (n, count) replacing (n, fields), fields taken in that order. prefetch > 0: that many host
    threads generate the next fields' hierarchies while the GPU trains on the current one."""
    import concurrent.futures as cf
    log = TrainLog()
    plan = [m for m, c in (sizes or [(n, fields)]) for _ in range(c)]
    fields = len(plan)
    total = max(1, fields * samples_per_field * steps_per_sample)
    t0 = time.time()
    step = 0
    specs = []
    for fi in range(fields):
        kw = dict(spec_kw or {})
        if identity_every and fi % identity_every == identity_every - 1:
            kw["coefficient"] = "identity"
        specs.append(FieldSpec(n=plan[fi], seed=seed0 + fi, **kw))
    ex = cf.ThreadPoolExecutor(prefetch) if prefetch > 0 else None
    futures = {}

    def ahead(i):
        if ex is not None:
            for j in range(i, min(fields, i + 2 * prefetch)):
                if j not in futures:
                    futures[j] = ex.submit(generate_field, specs[j], "sine", 2)

    for fi in range(fields):
        spec = specs[fi]
        ahead(fi)
        gen = futures.pop(fi).result() if fi in futures else None
        f = Field(spec, device=device, smoothers=smoothers, nu=nu, coarse_nu=coarse_nu, generated=gen)
        try:
            samples = make_samples(f, samples_per_field, seed=seed0 * 7919 + fi)
            for _ in range(steps_per_sample):
                for r, E, _e in samples:
                    cur = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * step / total))
                    loss, _ = net.train_step(f.ctx, r.data_ptr(), E, cur, weight_decay)
                    log.losses.append(loss)
                    step += 1
        finally:
            f.close()
        log.fields += 1
        if log_every and (fi + 1) % log_every == 0:
            recent = log.losses[-log_every * samples_per_field * steps_per_sample:]
            print(json.dumps({"fields": fi + 1, "mean_loss": float(np.mean(recent)),
                              "s": round(time.time() - t0, 1)}), flush=True)
    if ex is not None:
        ex.shutdown(wait=True, cancel_futures=True)
    log.steps = step
    log.seconds = time.time() - t0
    return log


def _cli():
    import argparse
    ap = argparse.ArgumentParser(description="train the learned correction step on the GPU")
    ap.add_argument("--fields", type=int, default=400)
    ap.add_argument("--n", type=int, default=16)
    ap.add_argument("--samples", type=int, default=4)
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--seed", type=int, default=1000)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--init", default="")
    ap.add_argument("--log-every", type=int, default=20)
    ap.add_argument("--nu", default="2,2", help="pre,post smoothing steps of the cycle the step corrects")
    ap.add_argument("--identity-every", type=int, default=4, help="every m-th field has K = I (0: none)")
    ap.add_argument("--coarse-nu", default="-1,-1", help="pre,post smoothing steps on levels >= 1 (-1: as --nu)")
    ap.add_argument("--sizes", default="", help="n:count,... fields per mesh size in order (replaces --n/--fields)")
    ap.add_argument("--prefetch", type=int, default=0, help="host threads generating the next fields ahead")
    a = ap.parse_args()
    nu = tuple(int(v) for v in a.nu.split(","))
    coarse_nu = tuple(int(v) for v in a.coarse_nu.split(","))
    net = N.Net(0)
    p0 = load_params(a.init)[0] if a.init else init_params(a.seed)
    net.set_params(p0)
    sizes = [tuple(int(v) for v in t.split(":")) for t in a.sizes.split(",")] if a.sizes else None
    log = train(net, fields=a.fields, n=a.n, samples_per_field=a.samples, steps_per_sample=a.repeat, lr=a.lr,
                seed0=a.seed, log_every=a.log_every, nu=nu, identity_every=a.identity_every, coarse_nu=coarse_nu,
                sizes=sizes, prefetch=a.prefetch)
    meta = {"fields": log.fields, "n": a.n if not sizes else {str(m): c for m, c in sizes}, "k": 1,
            "coefficient": "anisotropic diag(1,1,eps), eps log-U[1e-3,1], "
            "random rotation per 4^3 block" + (f"; every {a.identity_every}th field K = I" if a.identity_every else ""),
            "cycle": f"V({nu[0]},{nu[1]}) bgs/rbgs" + (f", V({coarse_nu[0]},{coarse_nu[1]}) on levels >= 1"
                                                       if min(coarse_nu) >= 0 else ""),
            "init": os.path.basename(a.init) if a.init else "random", "samples_per_field": a.samples, "repeat": a.repeat, "lr": a.lr,
            "seed0": a.seed, "steps": log.steps, "seconds": round(log.seconds, 1),
            "first_mean_loss": float(np.mean(log.losses[:200])) if log.losses else None,
            "final_mean_loss": float(np.mean(log.losses[-200:])) if log.losses else None}
    save_params(a.out, net.params(), meta)
    print(json.dumps(meta), flush=True)


if __name__ == "__main__":
    _cli()
