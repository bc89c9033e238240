"""CPU oracle of the learned correction step (TEST INFRASTRUCTURE ONLY).

The reference has no learned component: this file restates, in FP64 numpy, the network the GPU
library runs (fhhos4_gb300/csrc/fhg_learned.cu) so that its inputs, forward pass, energy loss and
gradients can be checked. It is imported by tests only; the product path never calls it.

Parity is therefore unpinned against the reference; the pins are
  * central finite differences of the exact FP64 loss (``exact=True``), and
  * the GPU's own rounding points mirrored here (``exact=False``): BF16 inputs, weights,
    activations (gelu in bf16 arithmetic, ``gelu_bf16``) and backpropagated signals, FP64
    accumulation in place of FP32; the backward pass uses the derivative of the exact gelu, as
    the GPU does.

Network (per face i; s_i, tensors and neighbour order as the GPU builds them):
    u = [w_i, w_j1..w_j6 (7 bs, zero padded to 32) / s_i, T1/tau, T2/tau, 0 0 0 0]   (48)
    a1 = W1 u + b1, h1 = gelu(a1); a2 = W2 h1 + b2, h2 = gelu(a2); y = W3 h2 + b3 (16)
    c_i = s_i y[:bs]
Loss of one field with error e, r = A e, E = e.r:  L = |e - c|_A^2 / E = 1 + (c.Ac - 2 c.r) / E.
"""
from __future__ import annotations

import numpy as np

K_IN, K_HID, K_OUT = 48, 128, 16
RESIDUAL_SLOTS, TENSOR_SLOTS, NEIGHBOURS = 32, 16, 6
OFF_W1 = 0
OFF_B1 = OFF_W1 + K_HID * K_IN
OFF_W2 = OFF_B1 + K_HID
OFF_B2 = OFF_W2 + K_HID * K_HID
OFF_W3 = OFF_B2 + K_HID
OFF_B3 = OFF_W3 + K_OUT * K_HID
N_PARAMS = OFF_B3 + K_OUT
GELU_C0 = np.sqrt(2.0 / np.pi)
GELU_C1 = 0.044715


def bf16(x) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def bf16_bits_to_float(bits) -> np.ndarray:
    b = np.asarray(bits, dtype=np.uint16).astype(np.uint32) << 16
    return b.view(np.float32).astype(np.float64)


def gelu(a):
    return 0.5 * a * (1.0 + np.tanh(GELU_C0 * (a + GELU_C1 * a ** 3)))


def gelu_bf16(a):
    """The activation as the GPU evaluates it (fhg_learned.cu: gelu_tanh_bf16x2, gelu_bf16x2):
    bf16 inputs, bf16x2 arithmetic (one rounding per multiply or FMA), tanh rounded to bf16 (the
    GPU's bf16x2 hardware tanh can differ in the last bit), result bf16:
    h + h tanh(x (c0 + c0 c1 x^2)), h = x / 2, with c0 and c0 c1 (an FP32 product) rounded to bf16."""
    x = bf16(a)
    c0 = bf16(np.float32(GELU_C0))
    c01 = bf16(np.float32(GELU_C0) * np.float32(GELU_C1))
    q = bf16(bf16(x * x) * c01 + c0)
    u = bf16(x * q)
    t = bf16(np.tanh(u))
    h = bf16(0.5 * x)
    return bf16(h * t + h)


def gelu_grad(a):
    t = np.tanh(GELU_C0 * (a + GELU_C1 * a ** 3))
    return 0.5 * (1.0 + t) + 0.5 * a * (1.0 - t * t) * GELU_C0 * (1.0 + 3.0 * GELU_C1 * a * a)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    W1 = p[OFF_W1:OFF_B1].reshape(K_HID, K_IN)
    b1 = p[OFF_B1:OFF_W2]
    W2 = p[OFF_W2:OFF_B2].reshape(K_HID, K_HID)
    b2 = p[OFF_B2:OFF_W3]
    W3 = p[OFF_W3:OFF_B3].reshape(K_OUT, K_HID)
    b3 = p[OFF_B3:N_PARAMS]
    return W1, b1, W2, b2, W3, b3


def pack(W1, b1, W2, b2, W3, b3) -> np.ndarray:
    return np.concatenate([W1.ravel(), b1, W2.ravel(), b2, W3.ravel(), b3])


def neighbours(A_bsr_rowptr, A_bsr_colidx, A_bsr_vals, bs):
    """Per block row: off-diagonal block columns by decreasing |A_ij|_F^2 rounded to FP32 (ties:
    smaller column), the first six, -1 padded (fhg_api.cu: learned_neighbours). vals: (nnzb, bs, bs)."""
    nb = len(A_bsr_rowptr) - 1
    key = np.sum(np.asarray(A_bsr_vals, dtype=np.float64).reshape(len(A_bsr_colidx), -1) ** 2, axis=1)
    key = key.astype(np.float32).astype(np.float64)
    out = -np.ones((nb, NEIGHBOURS), dtype=np.int64)
    for i in range(nb):
        row = []
        for p in range(A_bsr_rowptr[i], A_bsr_rowptr[i + 1]):
            j = int(A_bsr_colidx[p])
            if j != i:
                row.append((-key[p], j))
        row.sort()
        for k, (_, j) in enumerate(row[:NEIGHBOURS]):
            out[i, k] = j
    return out


def tensor_features(tensors) -> np.ndarray:
    """(nb, 12) element tensors -> (nb, 16) features: both divided by the larger Frobenius norm."""
    t = np.asarray(tensors, dtype=np.float64)
    out = np.zeros((t.shape[0], TENSOR_SLOTS))
    n0 = np.sqrt(np.sum(t[:, 0:3] ** 2, 1) + 2 * np.sum(t[:, 3:6] ** 2, 1))
    n1 = np.sqrt(np.sum(t[:, 6:9] ** 2, 1) + 2 * np.sum(t[:, 9:12] ** 2, 1))
    tau = np.maximum(n0, n1)
    ok = tau > 0
    out[ok, :12] = t[ok] / tau[ok, None]
    return bf16(out)


def features(nbr, w, tfeat, bs):
    """Input rows (nb, 48, BF16-rounded) and scales s (nb) from w = D^-1 r (nb*bs) and tensor features."""
    nb = nbr.shape[0]
    W = np.asarray(w, dtype=np.float64).reshape(nb, bs)
    v = np.zeros((nb, 7 * bs))
    v[:, :bs] = W
    for j in range(NEIGHBOURS):
        g = nbr[:, j]
        ok = g >= 0
        v[ok, (j + 1) * bs:(j + 2) * bs] = W[g[ok]]
    s = np.sqrt(np.mean(v * v, axis=1))
    inv = np.where(s > 0, 1.0 / np.where(s > 0, s, 1.0), 0.0)
    u = np.zeros((nb, K_IN))
    u[:, :7 * bs] = bf16(v * inv[:, None])
    u[:, RESIDUAL_SLOTS:] = tfeat
    return u, s


def forward(p, u, exact: bool = False):
    """Activations of every row of u: a1, h1, a2, h2, y (FP64; BF16 rounding points unless exact)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    rnd = (lambda x: x) if exact else bf16
    act = gelu if exact else gelu_bf16
    a1 = u @ rnd(W1).T + b1
    h1 = act(a1)
    a2 = h1 @ rnd(W2).T + b2
    h2 = act(a2)
    y = h2 @ rnd(W3).T + b3
    return a1, h1, a2, h2, y


def loss_and_grad(p, u, s, A, r, energy: float, bs: int, exact: bool = False):
    """Energy loss of one field and its gradient w.r.t. the parameters (flat, N_PARAMS).

    A: scipy sparse level-0 operator in the numbering of r (the GPU context's colour numbering),
    r = A e, energy = e.A e, u/s: the faces' inputs in the same numbering. With exact=False the
    signals fed back are rounded to BF16 where the GPU rounds them (dy, delta2, delta1)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    rnd = (lambda x: x) if exact else bf16
    a1, h1, a2, h2, y = forward(p, u, exact)
    nb = u.shape[0]
    r = np.asarray(r, dtype=np.float64)
    c = (s[:, None] * y[:, :bs]).ravel()
    q = A @ c
    loss = 1.0 + (np.dot(c, q) - 2.0 * np.dot(c, r)) / energy
    g = (-2.0 * (r - q) / energy).reshape(nb, bs)
    dy = np.zeros((nb, K_OUT))
    dy[:, :bs] = rnd(s[:, None] * g)
    dW3 = dy.T @ h2
    db3 = dy.sum(0)
    d2 = rnd((dy @ rnd(W3)) * gelu_grad(a2))
    dW2 = d2.T @ h1
    db2 = d2.sum(0)
    d1 = rnd((d2 @ rnd(W2)) * gelu_grad(a1))
    dW1 = d1.T @ u
    db1 = d1.sum(0)
    return loss, pack(dW1, db1, dW2, db2, dW3, db3)


def correction(p, u, s, bs, exact: bool = False):
    """c (nb*bs): the correction the network adds to x."""
    y = forward(p, u, exact)[4]
    return (s[:, None] * y[:, :bs]).ravel()
