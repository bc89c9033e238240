"""Learned correction step on the GPU: inputs, tensor-core forward and backward against the FP64
oracle (oracle/learned_oracle.py), training, the gain over the plain V-cycle, and the fallback rule."""
import math
import os

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from fhhos4_gb300 import _native as N  # noqa: E402
from fhhos4_gb300 import learned as LN  # noqa: E402
import learned_oracle as LO  # noqa: E402


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")


def _field(n=8, seed=3, **kw):
    return LN.Field(LN.FieldSpec(n=n, seed=seed, **kw))


def _permuted_operator(f):
    """Level-0 operator in the context's colour numbering, FP32-rounded values (the FP32 copy the
    GPU applies), as float64 CSR."""
    bs = f.bs
    idx = (f.perm[:, None].astype(np.int64) * bs + np.arange(bs)).ravel()
    A = f.As[0].tocsr()[idx][:, idx].tocsr()
    A32 = sp.csr_matrix((A.data.astype(np.float32).astype(np.float64), A.indices, A.indptr), shape=A.shape)
    return A, A32, idx


def _oracle_inputs(f, r):
    """Oracle features/scales for residual r (colour numbering) from its own restatement."""
    bs = f.bs
    A, A32, idx = _permuted_operator(f)
    B = A.tobsr(blocksize=(bs, bs))
    B.sort_indices()
    nbr = LO.neighbours(B.indptr, B.indices, B.data, bs)
    # D^-1 from the FP64 diagonal blocks, rounded to FP32 as the GPU's copy
    nb = f.nb
    Dinv = np.zeros((nb, bs, bs))
    for i in range(nb):
        for p in range(B.indptr[i], B.indptr[i + 1]):
            if B.indices[p] == i:
                Dinv[i] = np.linalg.inv(B.data[p])
    Dinv = Dinv.astype(np.float32).astype(np.float64)
    w = np.einsum("nij,nj->ni", Dinv, np.asarray(r, dtype=np.float64).reshape(nb, bs)).ravel()
    tfeat = LO.tensor_features(f.tensors[f.perm])
    u, s = LO.features(nbr, w, tfeat, bs)
    return u, s, A32


def _gpu_features(f, r):
    nb = f.nb
    feat = torch.empty(nb * LO.K_IN, dtype=torch.int16, device="cuda")
    scale = torch.empty(nb, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    f.ctx.learned_features(r.data_ptr(), feat.data_ptr(), scale.data_ptr())
    u = LO.bf16_bits_to_float(feat.cpu().numpy().view(np.uint16)).reshape(nb, LO.K_IN)
    return u, scale.cpu().numpy().astype(np.float64)


def _params_all_active(seed=5):
    p = LN.init_params(seed)
    rng = np.random.default_rng(seed + 1)
    p[LN.OFF_W3:LN.OFF_B3] = (rng.standard_normal(LN.OFF_B3 - LN.OFF_W3) * 0.1).astype(np.float32)
    p[LN.OFF_B1:LN.OFF_W2] = (rng.standard_normal(128) * 0.1).astype(np.float32)
    p[LN.OFF_B3:LN.N_PARAMS] = (rng.standard_normal(16) * 0.1).astype(np.float32)
    return p


def test_features_match_oracle():
    _need_gpu()
    f = _field(n=8, coefficient="anisotropic")
    try:
        (r, E, e), = LN.make_samples(f, 1, cycles=(1,), seed=11)
        u_g, s_g = _gpu_features(f, r)
        u_o, s_o, _ = _oracle_inputs(f, r.cpu().numpy())
        np.testing.assert_allclose(s_g, s_o, rtol=1e-5, atol=1e-30)
        # BF16 inputs: identical except where FP32/FP64 rounding differs across a BF16 boundary
        diff = np.abs(u_g - u_o)
        assert np.max(diff) <= 2.0 ** -7 * np.maximum(np.abs(u_o), 1e-3).max()
        assert np.mean(diff > 0) < 0.02
        assert np.array_equal(u_g[:, LO.RESIDUAL_SLOTS:], u_o[:, LO.RESIDUAL_SLOTS:])
    finally:
        f.close()


def test_gradient_matches_oracle():
    """Tensor-core forward + energy loss + backward (fhg_net_train_step, no update) against the FP64
    oracle with the GPU's BF16 rounding points, on the GPU's own inputs."""
    _need_gpu()
    f = _field(n=8, coefficient="anisotropic")
    net = N.Net(0)
    try:
        p = _params_all_active()
        net.set_params(p)
        (r, E, e), = LN.make_samples(f, 1, cycles=(2,), seed=12)
        loss_g, grad_g = net.train_step(f.ctx, r.data_ptr(), E, 0.0, update=False, want_grad=True)
        u, s = _gpu_features(f, r)
        _, A32, _ = _permuted_operator(f)
        loss_o, grad_o = LO.loss_and_grad(p, u, s, A32, r.cpu().numpy(), E, f.bs, exact=False)
        # tolerances: FP32 vs FP64 accumulation, and the hardware bf16x2 tanh of the activation,
        # which is an approximation (the oracle rounds the exact tanh to bf16)
        assert abs(loss_g - loss_o) <= 5e-3 * abs(loss_o) + 1e-6
        blocks = {"W1": (LN.OFF_W1, LN.OFF_B1), "b1": (LN.OFF_B1, LN.OFF_W2), "W2": (LN.OFF_W2, LN.OFF_B2),
                  "b2": (LN.OFF_B2, LN.OFF_W3), "W3": (LN.OFF_W3, LN.OFF_B3), "b3": (LN.OFF_B3, LN.N_PARAMS)}
        for name, (a, b) in blocks.items():
            go, gg = grad_o[a:b], grad_g[a:b].astype(np.float64)
            rel = np.linalg.norm(gg - go) / max(np.linalg.norm(go), 1e-30)
            assert rel < 3e-2, (name, rel)
        # the unused output rows (>= bs) get no gradient
        W3g = grad_g[LN.OFF_W3:LN.OFF_B3].reshape(16, 128)
        assert np.all(W3g[f.bs:] == 0)
        # parameters unchanged without update
        np.testing.assert_array_equal(net.params(), p)
    finally:
        net.close()
        f.close()


@pytest.mark.parametrize("kernel", ["tcgen05", "mma_sync"])
def test_fused_inference_matches_oracle(kernel):
    """The V-cycle with the learned step minus the plain V-cycle is exactly the correction of the
    fused kernel (tensor-memory tcgen05 tiles or mma.sync tiles); compare it with the oracle's
    forward pass on the same inputs."""
    _need_gpu()
    f = _field(n=8, coefficient="anisotropic")
    try:
        p = _params_all_active(7)
        f.ctx.set_learned(p, "always", kernel=kernel)
        (r, E, e), = LN.make_samples(f, 1, cycles=(1,), seed=13)
        z0 = torch.empty_like(r)
        z1 = torch.empty_like(r)
        f.vcycle(r, z0, learned=False)
        f.vcycle(r, z1, learned=True)
        c_gpu = (z1 - z0).cpu().numpy().astype(np.float64)
        # residual the step sees: r - A z0 (FP32 on the GPU)
        r1 = torch.empty_like(r)
        f.ctx.apply_internal(0, N.OP_RESIDUAL, "fp32", z0.data_ptr(), r.data_ptr(), r1.data_ptr())
        u, s = _gpu_features(f, r1)
        c_or = LO.correction(p, u, s, f.bs)
        rel = np.linalg.norm(c_gpu - c_or) / np.linalg.norm(c_or)
        assert rel < 1.5e-2, rel   # the hardware bf16x2 tanh vs the oracle's rounded exact tanh
    finally:
        f.close()


def test_tcgen05_and_mma_sync_kernels_agree_at_scale():
    """Both inference kernels on a 32^3 field (387,072 faces, every tile of both grids used)."""
    _need_gpu()
    f = _field(n=32, seed=21, coefficient="anisotropic")
    try:
        p = _params_all_active(9)
        (r, E, e), = LN.make_samples(f, 1, cycles=(1,), seed=14)
        z0 = torch.empty_like(r)
        f.vcycle(r, z0, learned=False)
        out = {}
        for kernel in ("tcgen05", "mma_sync"):
            f.ctx.set_learned(p, "always", kernel=kernel)
            z = torch.empty_like(r)
            f.vcycle(r, z, learned=True)
            out[kernel] = (z - z0).double()
        a, b = out["tcgen05"], out["mma_sync"]
        assert float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)) < 2e-3
    finally:
        f.close()


def test_training_reduces_loss_and_beats_plain_cycle():
    """Train briefly on seeded fields, then on a held-out field the learned V-cycle leaves less
    energy error than the plain one."""
    _need_gpu()
    net = N.Net(0)
    try:
        net.set_params(LN.init_params(0))
        log = LN.train(net, fields=12, n=8, samples_per_field=4, steps_per_sample=3, lr=3e-3, seed0=500)
        q = len(log.losses) // 4
        assert np.mean(log.losses[-q:]) < np.mean(log.losses[:q])
        assert np.mean(log.losses[-q:]) < 1.0
        f = _field(n=8, seed=9999, coefficient="anisotropic")
        try:
            f.ctx.set_learned(net.params(), "always")
            ratios = []
            for r, E, e in LN.make_samples(f, 3, cycles=(1, 2, 3), seed=77):
                ratios.append((LN.energy_ratio(f, e, False), LN.energy_ratio(f, e, True)))
            plain, learned = np.mean(ratios, axis=0)
            assert learned < plain, (plain, learned)
        finally:
            f.close()
    finally:
        net.close()


def _solve(f, mode, params=None, maxit=200):
    b = f.b
    if mode == "off":
        f.ctx.set_learned(None, "off")
    else:
        f.ctx.set_learned(params, mode)
    rc, x, hist, info = f.ctx.solve(b, maxit)
    return rc, x, hist, info


def test_learned_solve_reaches_fp64_tolerance():
    _need_gpu()
    net = N.Net(0)
    f = _field(n=16, seed=4242, coefficient="anisotropic")
    try:
        net.set_params(LN.init_params(0))
        LN.train(net, fields=6, n=8, samples_per_field=4, steps_per_sample=2, lr=3e-3, seed0=600)
        p = net.params()
        rc0, x0, h0, i0 = _solve(f, "off")
        assert rc0 == 0 and i0.true_relative_residual < 1e-8
        for mode in ("always", "fallback"):
            rc, x, h, info = _solve(f, mode, p)
            assert rc == 0
            assert h[-1] < 1e-8
            # the FP64 true residual judges the solve
            r_true = np.linalg.norm(f.b - f.As[0] @ x) / np.linalg.norm(f.b)
            assert info.true_relative_residual == pytest.approx(r_true, rel=1e-6)
            assert r_true < 1e-8 * (1 + 1e-6)
            assert 0 < info.learned_iterations <= info.iterations
            if mode == "always":
                assert info.learned_iterations == info.iterations
    finally:
        f.close()
        net.close()


def test_fallback_to_plain_cycle():
    """A network that spoils the cycle (large random output layer) is dropped by the fallback rule
    within a few iterations, and the solve still converges."""
    _need_gpu()
    f = _field(n=16, seed=4243, coefficient="anisotropic")
    try:
        rc0, _, h0, i0 = _solve(f, "off")
        bad = LN.init_params(1)
        rng = np.random.default_rng(3)
        bad[LN.OFF_W3:LN.OFF_B3] = (rng.standard_normal(LN.OFF_B3 - LN.OFF_W3) * 5.0).astype(np.float32)
        rc, x, h, info = _solve(f, "fallback", bad)
        assert rc == 0 and h[-1] < 1e-8
        assert info.learned_iterations < info.iterations
        assert info.learned_iterations <= 7   # the rule looks back four iterations from the sixth
        rho = f.ctx.learned_reference_rate()
        assert 0.0 < rho < 1.0
    finally:
        f.close()


def test_learned_requires_fp32_setup():
    _need_gpu()
    from fhhos4_gb300 import hho
    As, Ps, b, bs = hho.generate(3, 4, 1)
    ctx = N.Context(0)
    for l, A in enumerate(As):
        ctx.set_level(l, bs, A)
    for l, P in enumerate(Ps):
        ctx.set_prolongation(l, P)
    ctx.setup(len(As), N.default_options())  # FP64 V-cycle
    with pytest.raises(N.FhgError) as ei:
        ctx.set_learned(LN.init_params(0), "fallback")
    assert ei.value.code == N.FHG_ERR_UNSUPPORTED
    with pytest.raises(N.FhgError):
        ctx.set_learned(np.zeros(10, np.float32), "off")
    ctx.close()
