"""Train the learned initial guess on the device and write its parameters.

    python -m baorec.train_guess --steps 2000 --out baorec.jl_gb300/weights/guess_lightcone.npy

(run with baorec.jl_gb300 on sys.path).  Training pairs are 128^3 sub-boxes,
at the cell size of the 256^3 lightcone workload, of synthetic lognormal
fields in that workload's survey window (shell 1000-1500 Mpc/h, RA 0-90 deg,
Dec 0-45 deg), solved to 5e-7 by the residual-driven solver; the loss is the
mean squared Laplacian of the potential error.  Prints the loss history in
tenths and the held-out start residuals (FFT start vs learned start).
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import _lib, guess


def training_context(n_train: int = 128, mesh: int = 256, bias=2.0, f=0.8, R=15.0) -> tuple:
    bmin, side, cell = guess.lightcone_region(mesh)
    c = _lib.default_config()
    c.method = _lib.MULTIGRID
    c.mg_mode = _lib.MG_CONVERGENT
    for a in range(3):
        c.n[a] = n_train
        c.box_size[a] = n_train * cell
        c.box_min[a] = float(bmin[a])
    c.bias, c.f, c.smoothing_radius = bias, f, R
    ctx = _lib.Context(c)
    cfg = guess.TrainConfig(region_min=tuple(float(v) for v in bmin), region_size=(side, side, side))
    return ctx, cfg


def held_out(ctx, cfg, count=8, offset=10_000_000):
    """[(FFT-start residual, learned-start residual)] on unseen training-style fields."""
    import torch
    n3 = ctx.cfg.n[0] * ctx.cfg.n[1] * ctx.cfg.n[2]
    f = torch.empty(n3, device="cuda")
    phi = torch.empty(n3, device="cuda")
    out = []
    for i in range(count):
        guess.sample(ctx, cfg, offset + i, f.data_ptr(), phi.data_ptr())
        out.append((guess.start_residual(ctx, f.data_ptr(), "spectral"),
                    guess.start_residual(ctx, f.data_ptr(), "learned")))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--n", type=int, default=128)
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    ctx, cfg = training_context(a.n)
    cfg.steps, cfg.batch, cfg.lr, cfg.seed = a.steps, a.batch, a.lr, a.seed + 1000
    guess.init(ctx, a.seed)
    before = held_out(ctx, cfg)
    t0 = time.time()
    hist = guess.train(ctx, cfg)
    dt = time.time() - t0
    after = held_out(ctx, cfg)
    p = guess.get_params(ctx)
    if a.out:
        guess.save(a.out, p)
    print(json.dumps({
        "steps": a.steps, "batch": a.batch, "lr": a.lr, "train_seconds": dt,
        "loss_tenths": [float(np.mean(h)) for h in np.array_split(hist, 10)] if len(hist) >= 10 else hist.tolist(),
        "held_out_untrained": before, "held_out_trained": after,
        "mean_ratio_learned_over_fft": float(np.mean([b / a_ for a_, b in after])),
    }), flush=True)


if __name__ == "__main__":
    main()
