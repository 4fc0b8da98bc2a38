"""CPU restatement of the learned gas-optics network and its gradients.

Test infrastructure only (the checker of the GPU training kernels): nothing
in the product path imports it.  The network is the one the library trains
(9 features padded to 16 -> 128 -> 128 -> 128 -> 288, SiLU), stored as the
library's parameter blob (W1[16][128] b1 W2[128][128] b2 W3[128][128] b3
W4[128][288] b4).

Two versions of the same mathematics:

* ``forward_backward(..., emulate=True)`` follows the GPU kernels' number
  formats step by step -- bf16 weights, inputs, pre-activations, activations
  and output gradients, fp32 sums, the mean-square loss of the 280 live
  outputs -- so that the GPU gradients can be compared element by element;
* ``emulate=False`` is the same network in plain float64, whose analytic
  gradients ``finite_difference`` checks by central differences.
"""
from __future__ import annotations

import numpy as np

KIN, H, NOUT, NOUTP = 16, 128, 280, 288
OFF = {}
_o = 0
for _name, _size in (("W1", KIN * H), ("b1", H), ("W2", H * H), ("b2", H), ("W3", H * H), ("b3", H),
                     ("W4", H * NOUTP), ("b4", NOUTP)):
    OFF[_name] = (_o, _size)
    _o += _size
NPARAM = _o
SHAPES = {"W1": (KIN, H), "W2": (H, H), "W3": (H, H), "W4": (H, NOUTP), "b1": (H,), "b2": (H,), "b3": (H,),
          "b4": (NOUTP,)}


def unpack(p: np.ndarray) -> dict:
    return {k: p[o:o + n].reshape(SHAPES[k]) for k, (o, n) in OFF.items()}


def pack(d: dict) -> np.ndarray:
    p = np.zeros(NPARAM, dtype=np.float64)
    for k, (o, n) in OFF.items():
        p[o:o + n] = np.asarray(d[k], dtype=np.float64).reshape(-1)
    return p


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def loss_weights(w: np.ndarray | None = None) -> np.ndarray:
    out = np.zeros(NOUTP)
    out[:NOUT] = 1.0 if w is None else w[:NOUT]
    return out


def forward_backward(params: np.ndarray, x: np.ndarray, t: np.ndarray, w: np.ndarray | None = None,
                     emulate: bool = True):
    """Loss and gradient (blob order) of L = sum_j w_j (y_j - t_j)^2 / (rows * 280).

    x: (rows, 16) standardised inputs; t: (rows, 288) standardised targets."""
    P = unpack(np.asarray(params, dtype=np.float64))
    wj = loss_weights(w)
    rows = x.shape[0]
    if emulate:
        f = np.float32
        Wq = {k: bf16(P[k].astype(f)) for k in ("W1", "W2", "W3", "W4")}
        bq = {k: P[k].astype(f) for k in ("b1", "b2", "b3", "b4")}
        a = bf16(np.asarray(x, dtype=f))
        acts, zs = [a], []
        for l in (1, 2, 3):
            z = a @ Wq[f"W{l}"] + bq[f"b{l}"]
            zs.append(bf16(z))
            a = bf16(silu(z))
            acts.append(a)
        y = a @ Wq["W4"] + bq["b4"]
        e = (y - t.astype(f)) * (wj > 0)
        loss = float(np.sum(wj * e.astype(np.float64) ** 2) / (rows * NOUT))
        dz = bf16(2.0 * wj.astype(f) * e / f(rows * NOUT))
        g = {}
        for l in (4, 3, 2, 1):
            g[f"W{l}"] = acts[l - 1].T.astype(np.float64) @ dz.astype(np.float64)
            g[f"b{l}"] = dz.astype(np.float64).sum(axis=0)
            if l > 1:
                da = dz @ Wq[f"W{l}"].T
                dz = bf16(da * dsilu(zs[l - 2].astype(f)))
        return loss, pack(g)
    a = np.asarray(x, dtype=np.float64)
    acts, zs = [a], []
    for l in (1, 2, 3):
        z = a @ P[f"W{l}"] + P[f"b{l}"]
        zs.append(z)
        a = silu(z)
        acts.append(a)
    y = a @ P["W4"] + P["b4"]
    e = (y - t) * (wj > 0)
    loss = float(np.sum(wj * e ** 2) / (rows * NOUT))
    dz = 2.0 * wj * e / (rows * NOUT)
    g = {}
    for l in (4, 3, 2, 1):
        g[f"W{l}"] = acts[l - 1].T @ dz
        g[f"b{l}"] = dz.sum(axis=0)
        if l > 1:
            dz = (dz @ P[f"W{l}"].T) * dsilu(zs[l - 2])
    return loss, pack(g)


def finite_difference(params: np.ndarray, x: np.ndarray, t: np.ndarray, idx: np.ndarray, h: float = 1e-6) -> np.ndarray:
    """Central differences of the float64 loss w.r.t. the parameters at idx."""
    out = np.zeros(len(idx))
    p = np.asarray(params, dtype=np.float64).copy()
    for n, i in enumerate(idx):
        old = p[i]
        p[i] = old + h
        lp, _ = forward_backward(p, x, t, emulate=False)
        p[i] = old - h
        lm, _ = forward_backward(p, x, t, emulate=False)
        p[i] = old
        out[n] = (lp - lm) / (2 * h)
    return out
