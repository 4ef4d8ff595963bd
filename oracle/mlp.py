"""CPU oracle of the learned block ordering's collision predictor (test infrastructure only).

The reference has no learned component, so there is no reference code to follow here: this is a
float64 numpy restatement of the network the library trains on the GPU (sin/cos features ->
256 -> 256 -> 1, ReLU, binary cross-entropy on the logit), used by the tests to check the GPU's
forward pass, its gradients and its training.  With ``bf16_points=True`` it rounds where
the GPU kernels hold BF16 values (weights fed to the tensor cores, the activations H1 and H2,
the back-propagated dH2 and dH1), so a correct GPU pass agrees with it to FP32 accumulation
error; with ``bf16_points=False`` it is plain float64 and serves the finite-difference check.

Parameters are one flat float32 vector in the library's order: W1 [256][kin], b1 [256],
W2 [256][256], b2 [256], w3 [256], b3 [1].
"""
from __future__ import annotations

import numpy as np

HIDDEN = 256


def kin_of(dim: int) -> int:
    return ((2 * dim + 15) // 16) * 16


def param_count(dim: int) -> int:
    k = kin_of(dim)
    return HIDDEN * k + HIDDEN + HIDDEN * HIDDEN + HIDDEN + HIDDEN + 1


def split(params: np.ndarray, dim: int) -> dict:
    k = kin_of(dim)
    sizes = [("W1", (HIDDEN, k)), ("b1", (HIDDEN,)), ("W2", (HIDDEN, HIDDEN)), ("b2", (HIDDEN,)),
             ("w3", (HIDDEN,)), ("b3", (1,))]
    out, o = {}, 0
    for name, shape in sizes:
        n = int(np.prod(shape))
        out[name] = params[o:o + n].reshape(shape)
        o += n
    return out


def bf16(x) -> np.ndarray:
    """Round float32 values to BF16 (round to nearest, ties to even), returned as float32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def features(q: np.ndarray, dim: int) -> np.ndarray:
    """sin, cos of each joint, zero-padded to kin columns (float32)."""
    q = np.asarray(q, np.float32)
    x = np.zeros((len(q), kin_of(dim)), np.float32)
    x[:, 0:2 * dim:2] = np.sin(q)
    x[:, 1:2 * dim:2] = np.cos(q)
    return x


def forward(params: np.ndarray, x: np.ndarray, dim: int, bf16_points: bool = True) -> dict:
    """x: [n][kin] features (already BF16 values when bf16_points).  Returns the activations."""
    P = split(np.asarray(params, np.float32 if bf16_points else np.float64), dim)
    r = bf16 if bf16_points else (lambda v: np.asarray(v, np.float64))
    f32 = (lambda v: np.asarray(v, np.float32)) if bf16_points else (lambda v: np.asarray(v, np.float64))
    W1, W2 = r(P["W1"]).astype(np.float64), r(P["W2"]).astype(np.float64)
    x = np.asarray(x, np.float64)
    h1 = r(np.maximum(f32(x @ W1.T) + f32(P["b1"]), 0)).astype(np.float64)
    h2 = r(np.maximum(f32(h1 @ W2.T) + f32(P["b2"]), 0)).astype(np.float64)
    z = h2 @ P["w3"].astype(np.float64) + float(P["b3"][0])
    return {"x": x, "h1": h1, "h2": h2, "z": z, "p": 1.0 / (1.0 + np.exp(-z)), "W2": W2}


def loss_and_gradients(params: np.ndarray, x: np.ndarray, valid: np.ndarray, dim: int, bf16_points: bool = True):
    """Mean binary cross-entropy (label 1 = in collision = not valid) and its gradient."""
    P = split(np.asarray(params, np.float32 if bf16_points else np.float64), dim)
    f = forward(params, x, dim, bf16_points)
    n = len(x)
    y = 1.0 - np.asarray(valid, np.float64)
    z = f["z"]
    loss = float(np.mean(np.maximum(z, 0) - z * y + np.log1p(np.exp(-np.abs(z)))))
    r = bf16 if bf16_points else (lambda v: np.asarray(v, np.float64))
    f32 = (lambda v: np.asarray(v, np.float32)) if bf16_points else (lambda v: np.asarray(v, np.float64))
    dz = f32((f["p"] - y) / n).astype(np.float64)
    w3 = P["w3"].astype(np.float64)
    dh2 = r(np.where(f["h2"] > 0, f32(dz[:, None] * w3[None, :]), 0)).astype(np.float64)
    g1 = f32(dh2 @ f["W2"])
    dh1 = r(np.where(f["h1"] > 0, g1, 0)).astype(np.float64)
    grads = {
        "W1": dh1.T @ f["x"],
        "b1": dh1.sum(0),
        "W2": dh2.T @ f["h1"],
        "b2": dh2.sum(0),
        "w3": f["h2"].T @ dz,
        "b3": np.array([dz.sum()]),
    }
    flat = np.concatenate([grads[k].ravel() for k in ("W1", "b1", "W2", "b2", "w3", "b3")])
    return loss, flat


def auc(scores: np.ndarray, positive: np.ndarray) -> float:
    """Area under the ROC curve (Mann-Whitney statistic with average ranks for ties)."""
    scores = np.asarray(scores, np.float64)
    positive = np.asarray(positive, bool)
    order = np.argsort(scores, kind="mergesort")
    ranks = np.empty(len(scores), np.float64)
    s = scores[order]
    i = 0
    while i < len(s):
        j = i
        while j + 1 < len(s) and s[j + 1] == s[i]:
            j += 1
        ranks[order[i:j + 1]] = 0.5 * (i + j) + 1.0
        i = j + 1
    n_pos = int(positive.sum())
    n_neg = len(scores) - n_pos
    if n_pos == 0 or n_neg == 0:
        return float("nan")
    return float((ranks[positive].sum() - n_pos * (n_pos + 1) / 2.0) / (n_pos * n_neg))
