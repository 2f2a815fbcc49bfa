"""Seeded synthetic catalogs that stand in for the DESI UNIT mocks.

The reference measures on UNIT lightcone catalogs that are not available
here; these generators produce catalogs with the same shapes, sizes and value
distributions (FP32 SoA positions, unit weights):

* a lognormal galaxy field with target power spectrum
  ``P(k) = 2e4 (k / 0.1 h/Mpc)^-1.5 (Mpc/h)^3`` scaled by ``b²``, zero above
  the grid's Nyquist wave number (Gaussian field with ``ξ_G = ln(1+ξ)``,
  ``δ = exp(G - σ_G²/2) - 1``);
* particles drawn cell by cell with probability ∝ ``1 + δ`` (a Poisson
  sample conditioned on its total, so the count is exact), uniform inside
  each cell;
* lightcone shells ``r ∈ [r_min, r_max]`` over an RA/Dec patch seen from the
  origin, randoms uniform in volume (``∝ r² dr``), i.e. the same ``n(r)`` as
  the data.

Everything here is host-side input preparation (NumPy, untimed).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def _pk(k, amp=2.0e4, k0=0.1, slope=-1.5):
    out = np.zeros_like(k)
    m = k > 0
    out[m] = amp * (k[m] / k0) ** slope
    return out


def lognormal_field(n, L, bias=2.0, seed=0, amp=2.0e4):
    """Lognormal overdensity on an ``n³`` grid of side ``L`` (indexed [ix,iy,iz])."""
    rng = np.random.default_rng(seed)
    kf = 2 * np.pi / L
    k1 = np.fft.fftfreq(n, d=1.0 / n) * kf
    kr = np.fft.rfftfreq(n, d=1.0 / n) * kf
    kmag = np.sqrt(k1[:, None, None] ** 2 + k1[None, :, None] ** 2 + kr[None, None, :] ** 2)
    knyq = np.pi * n / L
    pk = bias * bias * _pk(kmag, amp)
    pk[kmag > knyq] = 0.0
    vol = L ** 3
    cellv = vol / n ** 3
    # ξ on the grid: ξ(r) = (1/V) Σ_k P(k) e^{ikr}
    xi = np.fft.irfftn(pk / vol, s=(n, n, n), axes=(0, 1, 2)) * n ** 3
    xig = np.log1p(np.clip(xi, -0.99, None))
    pg = np.fft.rfftn(xig).real * vol / n ** 3
    pg = np.clip(pg, 0.0, None)
    pg[kmag > knyq] = 0.0
    # Gaussian field with power pg: Fourier amplitudes from white noise
    white = rng.standard_normal((n, n, n))
    wk = np.fft.rfftn(white)
    gk = wk * np.sqrt(pg / cellv)
    g = np.fft.irfftn(gk, s=(n, n, n), axes=(0, 1, 2))
    sig2 = g.var()
    delta = np.exp(g - sig2 / 2.0) - 1.0
    return delta  # indexed [a,b,c] with the last axis halved in k; isotropic, so axis order is immaterial


def _sample_cells(prob, n_part, n, L, origin, rng):
    """Draw exactly ``n_part`` points with cell probabilities ``prob``."""
    p = prob.ravel()
    p = p / p.sum()
    counts = rng.multinomial(n_part, p)
    cells = np.repeat(np.arange(p.size), counts)
    ix, iy, iz = np.unravel_index(cells, (n, n, n))
    cell = L / n
    u = rng.random((3, n_part))
    x = origin[0] + (ix + u[0]) * cell
    y = origin[1] + (iy + u[1]) * cell
    z = origin[2] + (iz + u[2]) * cell
    perm = rng.permutation(n_part)
    return x[perm], y[perm], z[perm]


def field_cdf(delta):
    """Cumulative cell distribution ∝ 1 + δ of a field, for :func:`sample_field`."""
    w = np.clip(1.0 + delta, 0.0, None).ravel()
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    return cdf


def sample_field(delta, n_part, L, rng, shift=(0, 0, 0), cdf=None):
    """``n_part`` FP32 positions in the periodic box [0, L)^3 drawn from the
    cells of ``delta`` (indexed [ix, iy, iz]) with probability ∝ 1 + δ and
    uniform inside the cell, the field moved periodically by ``shift`` cells.
    The cells come from the inverse of the cumulative distribution, which is
    the same multinomial draw as :func:`_sample_cells` for many catalogs of
    one field without redoing its O(cells) work per catalog."""
    n = delta.shape[0]
    if cdf is None:
        cdf = field_cdf(delta)
    cells = np.searchsorted(cdf, rng.random(n_part), side="right")
    cells = np.minimum(cells, cdf.size - 1)
    ix, iy, iz = np.unravel_index(cells, delta.shape)
    cell = L / n
    u = rng.random((3, n_part))
    f32 = np.float32
    out = []
    for idx, sh, uu in ((ix, shift[0], u[0]), (iy, shift[1], u[1]), (iz, shift[2], u[2])):
        a = np.mod((idx + sh + uu) * cell, L).astype(f32)
        a[a >= f32(L)] = f32(0)
        out.append(a)
    return out


@dataclass
class BoxMock:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    w: np.ndarray
    box_size: np.ndarray
    box_min: np.ndarray


def box_mock(n_part=200_000, L=1000.0, n_grid=128, bias=2.0, seed=1234) -> BoxMock:
    """Periodic-box catalog: ``n_part`` FP32 particles Poisson-sampled from a
    lognormal field on an ``n_grid³`` grid of side ``L``, positions in [0, L)."""
    rng = np.random.default_rng(seed + 1)
    delta = lognormal_field(n_grid, L, bias=bias, seed=seed)
    x, y, z = _sample_cells(1.0 + delta, n_part, n_grid, L, (0.0, 0.0, 0.0), rng)
    f32 = np.float32
    x, y, z = (np.mod(a, L).astype(f32) for a in (x, y, z))
    # FP32 rounding may land exactly on L; keep every coordinate in [0, L)
    for a in (x, y, z):
        a[a >= f32(L)] = f32(0)
    return BoxMock(x, y, z, np.ones(n_part, f32),
                   np.full(3, L, f32), np.zeros(3, f32))


def _shell_uniform(n, r_min, r_max, ra_max_deg, dec_max_deg, rng):
    u = rng.random(n)
    r = (r_min ** 3 + u * (r_max ** 3 - r_min ** 3)) ** (1.0 / 3.0)
    ra = rng.random(n) * math.radians(ra_max_deg)
    sdec = rng.random(n) * math.sin(math.radians(dec_max_deg))
    cdec = np.sqrt(1.0 - sdec ** 2)
    return r * cdec * np.cos(ra), r * cdec * np.sin(ra), r * sdec


def _in_shell(x, y, z, r_min, r_max, ra_max_deg, dec_max_deg):
    r = np.sqrt(x * x + y * y + z * z)
    ra = np.arctan2(y, x)
    dec = np.arcsin(np.clip(z / np.maximum(r, 1e-30), -1, 1))
    return ((r >= r_min) & (r <= r_max) & (ra >= 0) & (ra <= math.radians(ra_max_deg))
            & (dec >= 0) & (dec <= math.radians(dec_max_deg)))


@dataclass
class LightconeMock:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    w: np.ndarray
    rx: np.ndarray
    ry: np.ndarray
    rz: np.ndarray
    rw: np.ndarray


def lightcone_mock(n_data=500_000, rand_factor=10, r_min=1000.0, r_max=1500.0,
                   ra_max=90.0, dec_max=45.0, n_grid=256, bias=2.0, seed=4321) -> LightconeMock:
    """Lightcone shell catalog seen from the origin: data Poisson-sampled from a
    lognormal field (grid ``n_grid³`` over the shell's bounding cube) and
    restricted to the exact shell; randoms ``rand_factor`` times as many,
    uniform in the same volume."""
    rng = np.random.default_rng(seed + 7)
    L = r_max * 1.02
    origin = (-0.01 * r_max, -0.01 * r_max, -0.01 * r_max)
    delta = lognormal_field(n_grid, L, bias=bias, seed=seed)
    cell = L / n_grid
    c = (np.arange(n_grid) + 0.5) * cell
    # cells whose centre lies inside a slightly enlarged shell
    pad = 1.8 * cell
    X = origin[0] + c[:, None, None]
    Y = origin[1] + c[None, :, None]
    Z = origin[2] + c[None, None, :]
    R = np.sqrt(X * X + Y * Y + Z * Z)
    near = (R >= r_min - pad) & (R <= r_max + pad) & (X >= -pad) & (Y >= -pad) & (Z >= -pad)
    prob = np.where(near, 1.0 + delta, 0.0)
    want = n_data
    xs, ys, zs = [], [], []
    got = 0
    while got < want:
        m = int((want - got) * 1.6) + 1000
        x, y, z = _sample_cells(prob, m, n_grid, L, origin, rng)
        keep = _in_shell(x, y, z, r_min, r_max, ra_max, dec_max)
        xs.append(x[keep]); ys.append(y[keep]); zs.append(z[keep])
        got += int(keep.sum())
    x = np.concatenate(xs)[:want]
    y = np.concatenate(ys)[:want]
    z = np.concatenate(zs)[:want]
    nr = n_data * rand_factor
    rx, ry, rz = _shell_uniform(nr, r_min, r_max, ra_max, dec_max, rng)
    f32 = np.float32
    return LightconeMock(x.astype(f32), y.astype(f32), z.astype(f32), np.ones(want, f32),
                         rx.astype(f32), ry.astype(f32), rz.astype(f32), np.ones(nr, f32))
