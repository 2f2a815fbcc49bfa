"""Learned initial guess of the residual-driven multigrid solve (no
reference counterpart): training, parameter files and evaluation through
the C ABI (``baorec_guess_*`` in include/baorec_gb300.h)."""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

from . import _lib

# survey window of the lightcone workload: shell 1000-1500 Mpc/h, RA 0-90 deg, Dec 0-45 deg
LIGHTCONE_WINDOW = dict(r_min=1000.0, r_max=1500.0, ra_min=0.0, ra_max=90.0, dec_min=0.0, dec_max=45.0)
WEIGHTS_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "weights")


@dataclass
class TrainConfig:
    steps: int = 500
    batch: int = 4
    lr: float = 1e-3
    seed: int = 1
    sigma_g: float = 0.6
    pk_slope: float = -1.5
    region_min: Sequence[float] = (0.0, 0.0, 0.0)
    region_size: Sequence[float] = (1.0, 1.0, 1.0)
    window: dict = field(default_factory=lambda: dict(LIGHTCONE_WINDOW))
    rtol: float = 5e-7
    loss: str = "laplacian"              # "mse" | "laplacian"

    def to_c(self) -> _lib.GuessTrainConfig:
        c = _lib.GuessTrainConfig()
        c.steps, c.batch, c.lr, c.seed = int(self.steps), int(self.batch), float(self.lr), int(self.seed)
        c.sigma_g, c.pk_slope = float(self.sigma_g), float(self.pk_slope)
        for a in range(3):
            c.region_min[a] = float(self.region_min[a])
            c.region_size[a] = float(self.region_size[a])
        for k in ("r_min", "r_max", "ra_min", "ra_max", "dec_min", "dec_max"):
            setattr(c, k, float(self.window[k]))
        c.rtol = float(self.rtol)
        c.loss = {"mse": 0, "laplacian": 1}[self.loss]
        return c


def num_params() -> int:
    return int(_lib.load().baorec_guess_num_params())


def init(ctx: _lib.Context, seed: int = 0):
    ctx.call("baorec_guess_init", int(seed))


def set_params(ctx: _lib.Context, params) -> None:
    p = np.ascontiguousarray(params, dtype=np.float32)
    ctx.call("baorec_guess_set_params", p.ctypes.data, p.size)


def get_params(ctx: _lib.Context) -> np.ndarray:
    p = np.zeros(num_params(), np.float32)
    ctx.call("baorec_guess_get_params", p.ctypes.data, p.size)
    return p


def train(ctx: _lib.Context, cfg: TrainConfig) -> np.ndarray:
    """Train the context's network on the device; returns the loss history."""
    hist = np.zeros(max(int(cfg.steps), 1), np.float32)
    c = cfg.to_c()
    ctx.call("baorec_guess_train", C.byref(c), hist.ctypes.data)
    return hist[: int(cfg.steps)]


def sample(ctx: _lib.Context, cfg: TrainConfig, index: int, f_ptr: int, phi_ptr: int) -> None:
    """One training pair into device meshes (moves the context's box)."""
    c = cfg.to_c()
    ctx.call("baorec_guess_sample", C.byref(c), int(index), f_ptr, phi_ptr)


def set_conv_path(ctx: _lib.Context, tensor_core: bool) -> None:
    """Run the covered 3x3x3 layers on the tcgen05 kernel (True, the default)
    or every layer on the mma.sync kernels (False)."""
    ctx.call("baorec_guess_set_conv_path", 1 if tensor_core else 0)


def tc_layers(ctx: _lib.Context) -> int:
    """Convolutions of the last network forward that ran on tcgen05."""
    return int(ctx.lib.baorec_guess_tc_layers(ctx.h))


def conv3(ctx: _lib.Context, x, w, bias=None, add=None, relu: bool = False, path: str = "tcgen05"):
    """One 3x3x3 zero-padded convolution of the network on CUDA tensors:
    x (n, n, n, cin) BF16 indexed [z, y, x, c]; w (27, cin, cout) FP32 with
    tap t = dx + 3 dy + 9 dz; bias (cout,) FP32; add (n, n, n, cout) BF16.
    Returns relu?(conv(x) + bias + add) as (n, n, n, cout) BF16.  path:
    "mma" (mma.sync), "tcgen05" (TMA slab loads, the network's path),
    "tcgen05_cpasync" (cp.async slab loads)."""
    import torch
    n, cin = int(x.shape[0]), int(x.shape[3])
    cout = int(w.shape[2])
    x = x.contiguous()
    w = w.to(torch.float32).contiguous()
    y = torch.empty((n, n, n, cout), dtype=torch.bfloat16, device=x.device)
    b = bias.to(torch.float32).contiguous() if bias is not None else None
    ad = add.contiguous() if add is not None else None
    ctx.call("baorec_guess_conv3", cin, cout, n, x.data_ptr(), w.data_ptr(), b.data_ptr() if b is not None else None,
             ad.data_ptr() if ad is not None else None, y.data_ptr(), 1 if relu else 0,
             {"mma": 0, "tcgen05": 1, "tcgen05_cpasync": 2}[path])
    return y


def save(path: str, params) -> None:
    np.save(path, np.asarray(params, np.float32))


def load_params(path: str) -> np.ndarray:
    p = np.load(path).astype(np.float32)
    if p.size != num_params():
        raise ValueError(f"{path}: {p.size} parameters, the network has {num_params()}")
    return p


def start_residual(ctx: _lib.Context, f_ptr: int, start: str) -> float:
    """Relative residual of the zero / FFT / learned start for the device rhs f."""
    r = C.c_double()
    ctx.call("baorec_start_residual", f_ptr, {"zero": 0, "spectral": 1, "learned": 2}[start], C.byref(r))
    return r.value


def lightcone_region(mesh: int = 256):
    """Box of the lightcone workload (survey bounding box plus a 25 Mpc/h pad):
    returns (box_min, side, cell) for a `mesh`^3 grid."""
    w = LIGHTCONE_WINDOW
    rmax = w["r_max"]
    lo = np.array([0.0, 0.0, 0.0])
    hi = np.array([rmax, rmax, rmax * np.sin(np.radians(w["dec_max"]))])
    pad = 25.0
    side = float(np.max(hi - lo) + pad)
    return lo - pad / 2, side, side / mesh
