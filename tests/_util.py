"""Shared helpers for the parity tests (inputs and comparisons)."""
import numpy as np

F32 = np.float32


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))


def uniform_box(n, L, seed, bmin=(0.0, 0.0, 0.0)):
    rng = np.random.default_rng(seed)
    pos = [(F32(bmin[a]) + rng.random(n).astype(F32) * F32(L)).astype(F32) for a in range(3)]
    for p in pos:
        p[p >= F32(bmin[0] + L)] = F32(bmin[0])
    w = (0.5 + rng.random(n)).astype(F32)
    return pos[0], pos[1], pos[2], w


def small_lightcone(n_data=20000, rand_factor=5, n_grid=32, seed=11):
    from baorec import mocks
    return mocks.lightcone_mock(n_data=n_data, rand_factor=rand_factor, n_grid=n_grid, seed=seed)


def to_np(t):
    try:
        return t.detach().cpu().numpy()
    except AttributeError:
        return np.asarray(t)
