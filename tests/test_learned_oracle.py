"""CPU checks of the learned-step oracle (oracle/learned_oracle.py) and of the parameter layout
shared with libfhg: the oracle is pinned by central finite differences of its exact FP64 loss,
since the reference has no learned component to compare with."""
import numpy as np
import pytest
import scipy.sparse as sp

from fhhos4_gb300 import _native as N
from fhhos4_gb300 import learned as LN
import learned_oracle as LO


def _problem(seed=0, nb=30, bs=3):
    rng = np.random.default_rng(seed)
    p = rng.standard_normal(LO.N_PARAMS) * 0.1
    u = rng.standard_normal((nb, LO.K_IN))
    s = rng.random(nb) + 0.5
    M = sp.random(nb * bs, nb * bs, density=0.1, random_state=seed + 1)
    A = (M @ M.T + sp.eye(nb * bs)).tocsr()
    e = rng.standard_normal(nb * bs)
    r = A @ e
    return p, u, s, A, r, float(e @ r), bs


def test_parameter_layout_matches_the_library():
    assert LO.N_PARAMS == N.LEARNED_PARAMS == LN.N_PARAMS == 24848
    assert (LO.OFF_W1, LO.OFF_B1, LO.OFF_W2, LO.OFF_B2, LO.OFF_W3, LO.OFF_B3) == \
        (LN.OFF_W1, LN.OFF_B1, LN.OFF_W2, LN.OFF_B2, LN.OFF_W3, LN.OFF_B3)


@pytest.mark.parametrize("seed", [0, 1])
def test_exact_gradient_matches_finite_differences(seed):
    p, u, s, A, r, E, bs = _problem(seed)
    L, g = LO.loss_and_grad(p, u, s, A, r, E, bs, exact=True)
    rng = np.random.default_rng(seed + 10)
    idx = np.concatenate([rng.choice(LO.N_PARAMS, 40, replace=False),
                          [LO.OFF_B1 + 1, LO.OFF_B2 + 2, LO.OFF_B3, LO.OFF_B3 + bs - 1]])
    h = 1e-6
    for i in idx:
        pp = p.copy(); pp[i] += h
        pm = p.copy(); pm[i] -= h
        fd = (LO.loss_and_grad(pp, u, s, A, r, E, bs, True)[0] - LO.loss_and_grad(pm, u, s, A, r, E, bs, True)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_zero_output_layer_is_the_plain_cycle():
    """With W3 = 0 and b3 = 0 the correction is zero and the loss is exactly 1 (no change)."""
    p, u, s, A, r, E, bs = _problem(2)
    p[LO.OFF_W3:] = 0.0
    L, g = LO.loss_and_grad(p, u, s, A, r, E, bs, exact=True)
    assert L == pytest.approx(1.0, abs=1e-15)
    assert np.all(g[:LO.OFF_W3] == 0)       # no signal reaches the hidden layers yet
    assert np.any(g[LO.OFF_W3:] != 0)


def test_outputs_beyond_the_block_size_get_no_gradient():
    p, u, s, A, r, E, bs = _problem(3)
    _, g = LO.loss_and_grad(p, u, s, A, r, E, bs)
    W3 = g[LO.OFF_W3:LO.OFF_B3].reshape(16, 128)
    assert np.all(W3[bs:] == 0) and np.all(g[LO.OFF_B3 + bs:] == 0)


def test_bf16_rounding_is_round_to_nearest_even():
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(0).standard_normal(10000).astype(np.float32) * 10.0 ** np.random.default_rng(1).integers(-8, 8, 10000)
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(LO.bf16(x), ref)


def test_features_are_scale_invariant_and_ordered():
    """u does not change when the residual is scaled by a > 0 and s scales with it (the correction is
    positively homogeneous); neighbours come by decreasing |A_ij|_F with ties by column."""
    rng = np.random.default_rng(4)
    bs, nb = 3, 50
    M = sp.random(nb * bs, nb * bs, density=0.05, random_state=5)
    A = (M + M.T + sp.eye(nb * bs) * 4).tocsr()
    B = A.tobsr(blocksize=(bs, bs))
    B.sort_indices()
    nbr = LO.neighbours(B.indptr, B.indices, B.data, bs)
    for i in range(nb):
        cols = [j for j in nbr[i] if j >= 0]
        assert i not in cols
        norms = []
        for j in cols:
            p = B.indptr[i] + list(B.indices[B.indptr[i]:B.indptr[i + 1]]).index(j)
            norms.append(np.float32(np.sum(B.data[p] ** 2)))
        assert all(norms[k] >= norms[k + 1] for k in range(len(norms) - 1))
    w = rng.standard_normal(nb * bs)
    tf = LO.tensor_features(rng.standard_normal((nb, 12)))
    u1, s1 = LO.features(nbr, w, tf, bs)
    u2, s2 = LO.features(nbr, 7.5 * w, tf, bs)
    np.testing.assert_array_equal(u1, u2)
    np.testing.assert_allclose(s2, 7.5 * s1, rtol=1e-14)


def test_tensor_features_normalised():
    t = np.zeros((3, 12))
    t[0, :3] = [2, 2, 2]           # 2 I
    t[0, 6:9] = [2e6, 2e6, 2e6]    # 2e6 I
    t[2, :6] = [1, 1, 1, 0.5, 0, 0]
    f = LO.tensor_features(t)
    assert f.shape == (3, 16)
    assert f[0, 6] == pytest.approx(1 / np.sqrt(3), rel=1e-2) and f[0, 0] == pytest.approx(1e-6 / np.sqrt(3), rel=1e-2)
    assert np.all(f[1] == 0)       # no tensors: zero features
    assert np.all(f[:, 12:] == 0)


def test_init_params_start_from_the_plain_cycle():
    p = LN.init_params(0)
    assert p.dtype == np.float32 and p.size == LN.N_PARAMS
    assert np.all(p[LN.OFF_W3:] == 0) and np.all(p[LN.OFF_B1:LN.OFF_W2] == 0)
    assert 0.1 < np.std(p[LN.OFF_W1:LN.OFF_B1]) < 0.3
