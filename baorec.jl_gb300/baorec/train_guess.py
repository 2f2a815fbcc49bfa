"""Train the learned initial guess on the device and write its parameters.

    python -m baorec.train_guess --steps 20000 --n 128 --mesh 128 \
        --out baorec.jl_gb300/weights/guess_lightcone.npy

(run with baorec.jl_gb300 on sys.path).  Training pairs are n^3 boxes at the
cell size of a mesh^3 grid over the lightcone workload's box (with n = mesh =
128 every pair covers the whole box at 11.9 Mpc/h: the first restriction of
the 256^3 workload, where guess_level 1 runs the network), filled with
synthetic lognormal fields in the survey window (shell 1000-1500 Mpc/h,
RA 0-90 deg, Dec 0-45 deg) and solved to 5e-7 by the residual-driven solver;
the loss is the mean squared Laplacian of the potential error, Adam at lr
1e-3, batch 4.  Training runs in chunks of --chunk steps (fresh fields in
every chunk, the Adam state carried over); after each chunk the parameters
are written to --checkpoints (if given) and the held-out start residuals
(FFT start vs learned start) are printed as one JSON line.
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
    ap.add_argument("--mesh", type=int, default=256, help="cell size of a mesh^3 grid over the workload box")
    ap.add_argument("--chunk", type=int, default=0, help="steps per chunk (0: one chunk)")
    ap.add_argument("--checkpoints", default=None, help="directory for the parameters after each chunk")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    ctx, cfg = training_context(a.n, a.mesh)
    cfg.batch, cfg.lr = a.batch, a.lr
    guess.init(ctx, a.seed)
    before = held_out(ctx, cfg)
    chunk = a.chunk if a.chunk > 0 else a.steps
    hist_all, done, t0 = [], 0, time.time()
    while done < a.steps:
        k = min(chunk, a.steps - done)
        cfg.steps, cfg.seed = k, a.seed + 1000 + done   # fresh fields in every chunk
        hist_all.append(guess.train(ctx, cfg))
        done += k
        after = held_out(ctx, cfg)
        if a.checkpoints:
            import os
            os.makedirs(a.checkpoints, exist_ok=True)
            guess.save(os.path.join(a.checkpoints, f"guess_step{done}.npy"), guess.get_params(ctx))
        print(json.dumps({"steps_done": done, "seconds": time.time() - t0, "loss": float(np.mean(hist_all[-1])),
                          "mean_ratio_learned_over_fft": float(np.mean([b / a_ for a_, b in after]))}), flush=True)
    dt = time.time() - t0
    hist = np.concatenate(hist_all)
    p = guess.get_params(ctx)
    if a.out:
        guess.save(a.out, p)
    print(json.dumps({
        "steps": a.steps, "batch": a.batch, "lr": a.lr, "n": a.n, "mesh": a.mesh, "train_seconds": dt,
        "loss_tenths": [float(np.mean(h)) for h in np.array_split(hist, 10)] if len(hist) >= 10 else hist.tolist(),
        "held_out_untrained": before, "held_out_trained": after,
        "mean_ratio_learned_over_fft": float(np.mean([b / a_ for a_, b in after])),
    }), flush=True)


if __name__ == "__main__":
    main()
