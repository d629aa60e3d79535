"""ORACLE — test infrastructure, never part of the product path.

CPU restatement (numpy) of the learned hit predictor's forward and backward
passes, used to check the gradients the tcgen05 kernels produce.  It follows
the same rounding points as the device code: fp16 embeddings and weights,
FP32 accumulation, hidden activations rounded to fp16 after bias + ReLU,
softmax cross-entropy gradient p - onehot rounded to fp16, backward
activations rounded to fp16 before the ReLU mask, all gradients summed (not
averaged) over the batch.  Parameter layout: include/crt.h
CRT_PREDICTOR_PARAMS, in the order W1[64][32], b1, W2[64][64], b2,
W3[128][64], b3, origin embedding [64^3][16], direction embedding [1024][16].
"""
from __future__ import annotations

import numpy as np

IN, HID, CLS, EMB, GRID, DBINS = 32, 64, 128, 16, 64, 32
N_EO, N_ED = GRID ** 3, DBINS * DBINS
oW1 = 0
oB1 = oW1 + HID * IN
oW2 = oB1 + HID
oB2 = oW2 + HID * HID
oW3 = oB2 + HID
oB3 = oW3 + CLS * HID
oEo = oB3 + CLS
oEd = oEo + N_EO * EMB
N_PARAMS = oEd + N_ED * EMB


def unpack(p):
    p = np.asarray(p, np.float32)
    return dict(W1=p[oW1:oB1].reshape(HID, IN), b1=p[oB1:oW2], W2=p[oW2:oB2].reshape(HID, HID), b2=p[oB2:oW3],
                W3=p[oW3:oB3].reshape(CLS, HID), b3=p[oB3:oEo], Eo=p[oEo:oEd].reshape(N_EO, EMB),
                Ed=p[oEd:].reshape(N_ED, EMB))


def ray_keys(rays, scene_min, scene_max):
    """Origin cell on the 64^3 grid of the scene box and the 32x32
    octahedral bin of the direction, in float32 as the kernel computes them."""
    f32 = np.float32
    o = rays[:, 0:3].astype(f32)
    d = rays[:, 4:7].astype(f32)
    mn = np.asarray(scene_min, f32)
    ext = np.maximum(np.asarray(scene_max, f32) - mn, f32(1e-20))
    s = (f32(GRID) / ext).astype(f32)
    c = np.floor(((o - mn).astype(f32) * s).astype(f32)).astype(np.int64)
    c = np.clip(c, 0, GRID - 1)
    cell = (c[:, 0] * GRID + c[:, 1]) * GRID + c[:, 2]
    a = (np.abs(d[:, 0]) + np.abs(d[:, 1])).astype(f32)
    a = (a + np.abs(d[:, 2])).astype(f32)
    with np.errstate(divide="ignore", invalid="ignore"):
        px = np.where(a > 0, (d[:, 0] / a).astype(f32), f32(0))
        py = np.where(a > 0, (d[:, 1] / a).astype(f32), f32(0))
    neg = d[:, 2] < 0
    qx = ((f32(1) - np.abs(py)).astype(f32) * np.where(px >= 0, f32(1), f32(-1))).astype(f32)
    qy = ((f32(1) - np.abs(px)).astype(f32) * np.where(py >= 0, f32(1), f32(-1))).astype(f32)
    px = np.where(neg, qx, px)
    py = np.where(neg, qy, py)
    bu = np.clip(((px + f32(1)).astype(f32) * f32(0.5 * DBINS)).astype(f32).astype(np.int64), 0, DBINS - 1)
    bv = np.clip(((py + f32(1)).astype(f32) * f32(0.5 * DBINS)).astype(f32).astype(np.int64), 0, DBINS - 1)
    return cell, bu * DBINS + bv


def _h(x):
    return np.asarray(x, np.float32).astype(np.float16).astype(np.float32)


def forward_backward(params, rays, targets, scene_min, scene_max):
    """Returns (gradient vector of N_PARAMS floats, summed loss, logits)."""
    P = unpack(params)
    W1, W2, W3 = _h(P["W1"]), _h(P["W2"]), _h(P["W3"])
    cell, dbin = ray_keys(rays, scene_min, scene_max)
    X = np.concatenate([_h(P["Eo"][cell]), _h(P["Ed"][dbin])], axis=1)
    H1 = _h(np.maximum(X @ W1.T + P["b1"], 0))
    H2 = _h(np.maximum(H1 @ W2.T + P["b2"], 0))
    L = (H2 @ W3.T + P["b3"]).astype(np.float32)
    m = L.max(axis=1, keepdims=True)
    e = np.exp((L - m).astype(np.float64))
    p = e / e.sum(axis=1, keepdims=True)
    t = np.asarray(targets, np.int64)
    loss = float(-(np.log(p[np.arange(len(t)), t])).sum())
    onehot = np.zeros_like(p)
    onehot[np.arange(len(t)), t] = 1
    G3 = _h(p - onehot)
    g = np.zeros(N_PARAMS, np.float64)
    g[oW3:oB3] = (G3.T.astype(np.float64) @ H2).reshape(-1)
    g[oB3:oEo] = G3.sum(axis=0)
    G2 = np.where(H2 > 0, _h(G3 @ W3), 0).astype(np.float32)
    g[oW2:oB2] = (G2.T.astype(np.float64) @ H1).reshape(-1)
    g[oB2:oW3] = G2.sum(axis=0)
    G1 = np.where(H1 > 0, _h(G2 @ W2), 0).astype(np.float32)
    g[oW1:oB1] = (G1.T.astype(np.float64) @ X).reshape(-1)
    g[oB1:oW2] = G1.sum(axis=0)
    dX = G1.astype(np.float64) @ W1
    dEo = np.zeros((N_EO, EMB))
    np.add.at(dEo, cell, dX[:, :EMB])
    dEd = np.zeros((N_ED, EMB))
    np.add.at(dEd, dbin, dX[:, EMB:])
    g[oEo:oEd] = dEo.reshape(-1)
    g[oEd:] = dEd.reshape(-1)
    return g.astype(np.float32), loss, L


BLOCKS = [("W1", oW1, oB1), ("b1", oB1, oW2), ("W2", oW2, oB2), ("b2", oB2, oW3), ("W3", oW3, oB3),
          ("b3", oB3, oEo), ("Eo", oEo, oEd), ("Ed", oEd, N_PARAMS)]
