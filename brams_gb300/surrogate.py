"""Training and evaluation of the learned gas optics on the GPU.

The network (include/gb_rrtmg_lw.h, gb_lw_mlp_*) is trained by the library's
own CUDA forward/backward/Adam kernels on layers that the library's plain
taumol produces for profiles of the synthetic generator widened to T noise
N(0, 10 K) and H2O x lognormal(0, 1.0).  The profiles mix the layer counts
and model tops of the solver's workloads (38 and 45 layers to 10 hPa, 60
layers to 5 hPa), so that the layer-thickness feature covers them.

PyTorch only holds device memory here; every computation is a library call.

    python -m brams_gb300.surrogate train --layers 8000000 --out brams_gb300/data/lw_mlp.gbmlp
"""
from __future__ import annotations

import argparse
import math
import os
import time

import numpy as np

from . import rrtmg_lw as R
from .profiles import ProfileSpec, make_state

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, "data", "lw_mlp.gbmlp")
TRAIN_SHAPES = [(45, 10.0), (38, 10.0), (60, 5.0)]  # (nlay, ptop hPa)
TRAIN_T_NOISE, TRAIN_H2O_SIGMA = 10.0, 1.0


def _torch():
    import torch

    return torch


def dev(a):
    """Fortran-ordered numpy array -> device tensor with the same memory order."""
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)).cuda()


class DeviceGrid:
    """One grid's rrtmg_lw inputs and outputs on the device (Fortran layouts)."""

    def __init__(self, st: dict, tauc: np.ndarray | None = None, mcica: bool = False):
        torch = _torch()
        self.ncol, self.nlay = st["play"].shape
        d = {k: dev(st[k]) for k in R.STATE_ORDER}
        d["tauaer"] = dev(st["tauaer"])
        for k in ("cldfrac", "ciwp", "clwp", "rei", "rel"):
            if k in st:
                d[k] = dev(st[k])
        if tauc is not None:
            d["tauc"] = dev(tauc)
        if mcica:
            for k in ("cldfmcl", "ciwpmcl", "clwpmcl", "taucmcl"):
                d[k] = torch.zeros((self.nlay, self.ncol, 140), dtype=torch.float64, device="cuda")
            d["reicmcl"] = torch.zeros((self.nlay, self.ncol), dtype=torch.float64, device="cuda")
            d["relqmcl"] = torch.zeros((self.nlay, self.ncol), dtype=torch.float64, device="cuda")
        for k in ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt"):
            d[k] = torch.zeros((self.nlay + 1, self.ncol), dtype=torch.float64, device="cuda")
        d["hr"] = torch.zeros((self.nlay, self.ncol), dtype=torch.float64, device="cuda")
        d["hrc"] = torch.zeros((self.nlay, self.ncol), dtype=torch.float64, device="cuda")
        self.d = d

    def desc(self, mode=R.CLOUD_FUSED, icld=3, seed0=0, **extra) -> R.GridDesc:
        arrays = dict(self.d)
        if mode == R.CLOUD_FUSED:
            arrays["reicmcl"], arrays["relqmcl"] = self.d.get("rei"), self.d.get("rel")
        arrays.update(extra)
        return R.grid_desc(self.ncol, self.nlay, arrays, icld=icld, cloud_mode=mode, seed0=seed0)

    def outputs(self) -> dict:
        return {k: self.d[k].cpu().numpy().T.copy() for k in
                ("uflx", "dflx", "uflxc", "dflxc", "duflx_dt", "duflxc_dt", "hr", "hrc")}


def make_samples(ctx: R.Context, mlp: R.Mlp, n_layers: int, seed: int = 7, chunk_cols: int = 16384):
    """Features, taug and Planck fractions of about n_layers layers from the plain taumol (device tensors)."""
    torch = _torch()
    per_shape = n_layers // len(TRAIN_SHAPES)
    feats, taus, fracs = [], [], []
    k = 0
    for nlay, ptop in TRAIN_SHAPES:
        cols = max(1, per_shape // nlay)
        done = 0
        while done < cols:
            n = min(chunk_cols, cols - done)
            spec = ProfileSpec(ncol=n, nlay=nlay, seed=seed * 1000 + k, ptop=ptop, t_noise=TRAIN_T_NOISE,
                               h2o_sigma=TRAIN_H2O_SIGMA)
            k += 1
            g = DeviceGrid(make_state(spec))
            rows = n * nlay
            f = torch.empty((rows, 9), dtype=torch.float32, device="cuda")
            t = torch.empty((rows, 140), dtype=torch.float32, device="cuda")
            p = torch.empty((rows, 140), dtype=torch.float32, device="cuda")
            mlp.samples(g.desc(icld=0), f, t, p)
            feats.append(f)
            taus.append(t)
            fracs.append(p)
            done += n
    torch.cuda.synchronize()
    return torch.cat(feats), torch.cat(taus), torch.cat(fracs)


def train(ctx: R.Context, n_layers: int = 8_000_000, epochs: int = 12, batch: int = 16384, lr: float = 2e-3,
          seed: int = 7, log=print, mlp: R.Mlp | None = None):
    """Trains a network on plain-taumol samples; returns (mlp, history)."""
    torch = _torch()
    t0 = time.time()
    mlp = mlp or R.Mlp(ctx, seed=seed)
    feat, tau, frac = make_samples(ctx, mlp, n_layers, seed=seed)
    rows = feat.shape[0]
    mlp.fit_norm(rows, feat, tau, frac)
    x = torch.empty((rows, 16), dtype=torch.bfloat16, device="cuda")
    t = torch.empty((rows, 288), dtype=torch.float32, device="cuda")
    mlp.prepare(rows, feat, tau, frac, x, t)
    del tau, frac
    torch.cuda.synchronize()
    t_data = time.time() - t0
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    steps_per_epoch = rows // batch
    total = epochs * steps_per_epoch
    hist = []
    step = 0
    t1 = time.time()
    for ep in range(epochs):
        perm = torch.randperm(rows, device="cuda", generator=g)
        acc = torch.zeros(1, dtype=torch.float32, device="cuda")
        for i in range(steps_per_epoch):
            idx = perm[i * batch:(i + 1) * batch]
            xb = x.index_select(0, idx)
            tb = t.index_select(0, idx)
            lr_s = 1e-5 + 0.5 * (lr - 1e-5) * (1.0 + math.cos(math.pi * step / max(1, total)))
            mlp.train_step(batch, xb, tb, lr_s, loss)
            acc += loss
            step += 1
        hist.append(float(acc.item()) / max(1, steps_per_epoch))
        log(f"epoch {ep + 1}/{epochs}: loss {hist[-1]:.5f} ({time.time() - t1:.1f} s)")
    torch.cuda.synchronize()
    info = {"rows": rows, "epochs": epochs, "batch": batch, "lr": lr, "data_s": t_data,
            "train_s": time.time() - t1, "loss": hist}
    return mlp, info


def load(ctx: R.Context, path: str = DEFAULT_WEIGHTS) -> R.Mlp:
    return R.Mlp(ctx, path=path)


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    tr = sub.add_parser("train")
    tr.add_argument("--layers", type=int, default=8_000_000)
    tr.add_argument("--epochs", type=int, default=12)
    tr.add_argument("--batch", type=int, default=16384)
    tr.add_argument("--lr", type=float, default=2e-3)
    tr.add_argument("--seed", type=int, default=7)
    tr.add_argument("--out", default=DEFAULT_WEIGHTS)
    a = ap.parse_args()
    ctx = R.Context()
    mlp, info = train(ctx, a.layers, a.epochs, a.batch, a.lr, a.seed)
    mlp.save(a.out)
    print({k: v for k, v in info.items() if k != "loss"}, "final loss", info["loss"][-1])


if __name__ == "__main__":
    main()
