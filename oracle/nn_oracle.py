"""CPU reference of the a-priori MLP gate: features, forward, loss, gradient.

TEST INFRASTRUCTURE ONLY: the checker for the BF16 tensor-core kernels of
gp-mood_gb300/csrc/nn_gate.cu.  Two gradients are provided:
  * ``loss_grad(..., emulate_bf16=True)`` rounds every matrix-product operand
    to BF16 exactly where the kernels do (inputs, weights, hidden activations,
    the backpropagated hidden gradients) and accumulates in float64, so the
    kernels must agree to accumulation-order rounding;
  * ``emulate_bf16=False`` is the plain FP64 gradient of the same network.
Parameter vector (PyTorch flatten order of nn.Linear layers): W0[64][36],
b0[64], W1[64][64], b1[64], w2[1][64], b2[1] -- the order the reference's
save_NN_for_fortran.py writes (neural_network/save_NN_for_fortran.py:13-23).
"""
from __future__ import annotations

import numpy as np

NIN, NH = 36, 64
NPARAMS = NH * NIN + NH + NH * NH + NH + NH + 1
OFFS = {"W0": 0, "b0": NH * NIN, "W1": NH * NIN + NH, "b1": NH * NIN + NH + NH * NH,
        "w2": NH * NIN + 2 * NH + NH * NH, "b2": NH * NIN + 3 * NH + NH * NH}

# 9-point radius-2 cross: (0,0), (-1,0), (1,0), (0,-1), (0,1), (-2,0), (2,0), (0,-2), (0,2)
CROSS = [(0, 0), (-1, 0), (1, 0), (0, -1), (0, 1), (-2, 0), (2, 0), (0, -2), (0, 2)]


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(p: np.ndarray, dtype=np.float32):
    p = np.asarray(p, dtype=dtype)
    W0 = p[OFFS["W0"]:OFFS["b0"]].reshape(NH, NIN)
    b0 = p[OFFS["b0"]:OFFS["W1"]]
    W1 = p[OFFS["W1"]:OFFS["b1"]].reshape(NH, NH)
    b1 = p[OFFS["b1"]:OFFS["w2"]]
    w2 = p[OFFS["w2"]:OFFS["b2"]]
    b2 = p[OFFS["b2"]]
    return W0, b0, W1, b1, w2, b2


def features(U: np.ndarray, lf: int, nf: int):
    """36 features per interior cell (x fastest) and constant-stencil flags."""
    ng = 4
    q = np.stack([U[ng + dy: ng + dy + nf, ng + dx: ng + dx + lf, :].astype(np.float32) for dx, dy in CROSS],
                 axis=-1)  # [nf, lf, 4, 9]
    mx, mn = q.max(axis=-1), q.min(axis=-1)
    am = np.abs(q).max(axis=-1)
    with np.errstate(over="ignore", invalid="ignore"):  # subnormal max-abs: 1/am = inf, as in FP32 on the GPU
        scale = np.where(am > 0, np.float32(1.0) / np.where(am > 0, am, 1), 0).astype(np.float32)
        x = (q * scale[..., None]).reshape(nf * lf, 36)
    cst = np.all((mx - mn) < np.float32(1e-10), axis=-1).reshape(-1)
    return x.astype(np.float32), cst


def _rounder(emulate_bf16):
    if emulate_bf16:
        return lambda a: bf16(np.asarray(a, dtype=np.float32)).astype(np.float64)
    return lambda a: np.asarray(a, dtype=np.float64)


def forward(p, x, emulate_bf16=True):
    W0, b0, W1, b1, w2, b2 = unpack(p, np.float32 if emulate_bf16 else np.float64)
    r = _rounder(emulate_bf16)
    x64 = r(x)
    a1 = x64 @ r(W0).T + b0
    h1 = np.maximum(a1, 0)
    a2 = r(h1) @ r(W1).T + b1
    h2 = np.maximum(a2, 0)
    z = r(h2) @ r(w2) + b2
    return z, (x64, a1, h1, a2, h2)


def softplus(z):
    return np.maximum(z, 0) + np.log1p(np.exp(-np.abs(z)))


def loss_grad(p, x, y, pos_weight=1.0, emulate_bf16=True):
    """Mean weighted BCE with logits and its gradient (float64)."""
    W0, b0, W1, b1, w2, b2 = unpack(p, np.float32 if emulate_bf16 else np.float64)
    r = _rounder(emulate_bf16)
    y = np.asarray(y, dtype=np.float64)
    n = len(y)
    z, (x64, a1, h1, a2, h2) = forward(p, x, emulate_bf16)
    loss = np.mean(pos_weight * y * softplus(-z) + (1 - y) * softplus(z))
    s = 1 / (1 + np.exp(-z))
    dz = (pos_weight * y * (s - 1) + (1 - y) * s) / n
    h2b = r(h2)
    g_w2 = dz @ h2b
    g_b2 = dz.sum()
    w2b = r(w2)
    dh2 = np.where(a2 > 0, dz[:, None] * w2b[None, :], 0.0)
    g_b1 = dh2.sum(axis=0)
    dh2b = r(dh2)
    h1b = r(h1)
    g_W1 = dh2b.T @ h1b
    dh1 = np.where(a1 > 0, dh2b @ r(W1), 0.0)
    g_b0 = dh1.sum(axis=0)
    dh1b = r(dh1)
    g_W0 = dh1b.T @ x64
    g = np.concatenate([g_W0.ravel(), g_b0, g_W1.ravel(), g_b1, g_w2, [g_b2]])
    return loss, g


# ---------------------------------------------------------------------------
# The reference's own network (mod_NN.f90:14-58,157-183, format_input of
# mod_append_NN_dataset.f90:81-125): raw FP32 conserved variables of the R+1
# stencil ixiy_sp1(Mord+2, :) (GP_init.f90:270-355), variable fastest; FP32
# sigmoid MLP; r(1) > r(2) -> CellGPO 1, else 3; constant stencils -> 3.
SP1 = [(0, 0), (-1, 0), (0, 1), (1, 0), (0, -1), (-1, -1), (-1, 1), (1, 1), (1, -1), (0, -2), (-2, 0), (0, 2), (2, 0),
       (-3, 0), (-2, 1), (-1, 2), (0, 3), (1, 2), (2, 1), (3, 0), (2, -1), (1, -2), (0, -3), (-1, -2), (-2, -1)]


def ref_features(U: np.ndarray, mord: int):
    """(x [nf*lf, L] float32, constant [nf*lf] bool) of every interior cell, x fastest."""
    npts = 13 if mord == 3 else 25
    nf, lf = U.shape[0] - 8, U.shape[1] - 8
    cols = []
    for ox, oy in SP1[:npts]:
        cols.append(U[4 + oy:4 + oy + nf, 4 + ox:4 + ox + lf].astype(np.float32).reshape(-1, 4))
    q = np.stack(cols, axis=1)  # [cells, npts, 4]
    span = q.max(axis=1) - q.min(axis=1)  # float32
    const = np.all(span.astype(np.float64) < 1e-10, axis=1)
    return q.reshape(q.shape[0], -1), const


def ref_unpack(p: np.ndarray, L: int):
    n = p.size
    length = next(k for k in range(1, 129) if k * k + (L + 4) * k + 2 == n)
    o = 0
    W0 = p[o:o + length * L].reshape(length, L); o += length * L
    b0 = p[o:o + length]; o += length
    W1 = p[o:o + length * length].reshape(length, length); o += length * length
    b1 = p[o:o + length]; o += length
    W2 = p[o:o + 2 * length].reshape(2, length); o += 2 * length
    b2 = p[o:o + 2]
    return W0, b0, W1, b1, W2, b2


def ref_forward(p: np.ndarray, x: np.ndarray):
    """r [cells, 2] of the reference's forward in FP32, sums in index order."""
    x = x.astype(np.float32)
    W0, b0, W1, b1, W2, b2 = ref_unpack(np.asarray(p, np.float32), x.shape[1])
    one = np.float32(1.0)

    def layer(W, b, h):
        s = np.zeros((h.shape[0], W.shape[0]), np.float32)
        for j in range(W.shape[1]):
            s = s + W[:, j][None, :] * h[:, j][:, None]
        return s + b[None, :]

    h0 = layer(W0, b0, x)
    h0 = one / (one + np.exp(-h0))
    h1 = layer(W1, b1, h0)
    h1 = one / (one + np.exp(-h1))
    return layer(W2, b2, h1)
