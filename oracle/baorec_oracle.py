"""CPU oracle for the BAO reconstruction hot path of BAOrec.jl (test infrastructure).

This module is the checker, never the product: only the tests, the smoke check
and the CPU-baseline leg of the benchmark import it.  It restates, in NumPy,
the reference's CPU algorithm function by function; each function cites the
Julia file:line it follows (paths inside the BAOrec.jl project).

Two arithmetic modes share one code path:
  * ``dtype=np.float32`` emulates the reference CPU path: FP32 storage and
    FP32 per-operation rounding in the reference's evaluation order wherever
    Julia fixes that order (paint indices/weights, read-out sums, k axes).
  * ``dtype=np.float64`` is the FP64 oracle used to quote the relative L2
    error of the displacement field.

Parity status: UNPINNED against the reference itself.  The reference is
Julia (no Julia toolchain here) and its only stored outputs
(``test/bchmk_*.csv``) were computed from catalogs that are not available, so
no golden vector of the reference can be reproduced.  The oracle is instead
pinned by analytic known-answer tests (single-particle paint, plane waves
through the k-space operators, manufactured multigrid solutions, mass
conservation) under ``tests/``.

Layout: every mesh is a NumPy array indexed ``[ix, iy, iz]`` (0-based; the
reference's ``ρ[ix+1, iy+1, iz+1]``).  The real-to-complex transform halves
axis 0 (x), as ``rfftfreq(dims[1])`` does in ``src/utils.jl:6``.
"""
from __future__ import annotations

import math
import numpy as np
import scipy.fft as sfft

__all__ = [
    "setup_box", "k_vec", "x_vec", "cic", "tsc", "read_cic", "smooth",
    "setup_overdensity", "setup_overdensity_randoms", "iterate",
    "reconstructed_overdensity", "compute_displacements_iterative",
    "compute_displacements_multigrid", "read_shifts", "reconstructed_positions",
    "jacobi", "residual", "prolong", "reduce", "vcycle", "fmg",
    "reconstructed_potential", "run_iterative", "run_multigrid",
    "cell_keys", "cell_counts", "stencil_coefficients", "apply_operator",
    "gauss_seidel_rb", "solve_mg", "rfft3", "irfft3",
]

_FFT_WORKERS = None  # scipy.fft worker count; None = single thread


def set_fft_workers(n):
    """Number of threads scipy.fft may use (CPU baseline timing only)."""
    global _FFT_WORKERS
    _FFT_WORKERS = n


# ----------------------------------------------------------------------------
# FFT helpers (FFTW in the reference, scipy.fft/pocketfft here)
# ----------------------------------------------------------------------------

def rfft3(a):
    """Forward real 3-D DFT, unnormalised, halving axis 0 (``plan_rfft``,
    ``src/recon.jl:36``).  FP32 input is transformed in single precision."""
    return sfft.rfftn(a, axes=(2, 1, 0), workers=_FFT_WORKERS)


def irfft3(ak, n1):
    """Normalised inverse of :func:`rfft3` (``ldiv!(x, plan, x_k)``,
    ``src/utils.jl:54``)."""
    return sfft.irfftn(ak, s=(ak.shape[2], ak.shape[1], n1), axes=(2, 1, 0),
                       workers=_FFT_WORKERS)


# ----------------------------------------------------------------------------
# Grid utilities — src/utils.jl
# ----------------------------------------------------------------------------

def setup_box(x, y, z, pad, dtype=np.float32):
    """Cubic box enclosing the points with ``pad`` added, ``src/utils.jl:100-109``.

    ``box_min = min - pad/2``; ``box_size`` is the largest extent of
    ``box_max - box_min`` (so the pad is included) on all three axes.
    """
    T = dtype
    pad = T(pad)
    half = T(pad / T(2))
    bmin = np.array([T(np.min(d)) - half for d in (x, y, z)], dtype=T)
    bmax = np.array([T(np.max(d)) + half for d in (x, y, z)], dtype=T)
    side = T(np.max(bmax - bmin))
    return np.array([side, side, side], dtype=T), bmin


def k_vec(dims, box_size, dtype=np.float32):
    """Wave-number axes, ``src/utils.jl:3-10``.

    ``sample_rate = T(2π·n/L)`` (computed in FP64, rounded to T); the axes are
    ``rfftfreq(n1, fs1)`` and ``fftfreq(n2|n3, fs)``, i.e. ``i · T(fs/n)`` with
    the negative half of ``fftfreq`` starting at ``-n/2``.
    """
    T = dtype
    out = []
    for a, n in enumerate(dims):
        fs = T(2.0 * math.pi * n / float(box_size[a]))
        mult = T(fs / T(n))
        if a == 0:
            idx = np.arange(n // 2 + 1)
        else:
            idx = np.arange(n)
            idx = np.where(idx < (n + 1) // 2, idx, idx - n)
        out.append(idx.astype(T) * mult)
    return tuple(out)


def x_vec(dims, box_size, box_min, dtype=np.float32):
    """Cell-centre coordinate axes, ``src/utils.jl:21-25``.

    ``box_min + (i + 1/2)·cell`` with ``cell = T(L/n)``; the range is built
    in FP64 and rounded to T, as the reference's ``collect`` of a Float64
    range followed by ``map(T, ...)`` does.
    """
    T = dtype
    out = []
    for a, n in enumerate(dims):
        cell = float(T(T(box_size[a]) / T(n)))
        v = float(box_min[a]) + (np.arange(n, dtype=np.float64) + 0.5) * cell
        out.append(v.astype(T))
    return tuple(out)


def _kk(k, shape_k):
    """Broadcastable k axes for a halved spectrum of shape (n1/2+1, n2, n3)."""
    kx, ky, kz = k
    return kx[:, None, None], ky[None, :, None], kz[None, None, :]


def _k2(k, T):
    kx, ky, kz = _kk(k, None)
    # k⃗[1]^2 + k⃗[2]^2 + k⃗[3]^2, left to right in T
    return (kx * kx + ky * ky) + kz * kz


def smooth(field, R, box_size):
    """Gaussian smoothing in k space, ``src/utils.jl:45-56``.

    ``δ_k = rfft(δ)``; ``δ_k *= exp(-0.5 R² k²)`` with the exponent evaluated
    in FP64 (the ``-0.5`` literal promotes it) and the product rounded back to
    the spectrum's precision; ``δ = irfft(δ_k)``.
    """
    T = field.dtype.type
    k = k_vec(field.shape, box_size, T)
    fk = rfft3(field)
    k2 = _k2(k, T)
    R2 = T(T(R) * T(R))
    fac = np.exp(-0.5 * float(R2) * k2.astype(np.float64))
    fk = (fk.astype(np.complex128) * fac).astype(fk.dtype)
    return irfft3(fk, field.shape[0]).astype(T)


# ----------------------------------------------------------------------------
# Mass assignment — src/mas.jl
# ----------------------------------------------------------------------------

def _grid_coord(p, bmin, L, n, T):
    """``(p - box_min)·n / box_size + 1`` in T, evaluated left to right with
    one rounding per operation (``src/mas.jl:13-15``)."""
    return (p.astype(T) - T(bmin)) * T(n) / T(L) + T(1)


def cic(rho, x, y, z, w, box_size, box_min, wrap=True):
    """Cloud-in-cell paint, ``src/mas.jl:1-52`` (CPU method).

    Accumulates into ``rho`` (not cleared) in particle order, exactly like the
    reference's serial loop.  Returns ``(rho, (x, y, z))`` where the positions
    are the wrapped copies the reference writes back into its inputs when
    ``wrap`` is set (``src/mas.jl:7-11``: every axis is tested against
    ``box_min[1]`` / ``box_size[1]``).

    Raises ``IndexError`` where the reference raises ``BoundsError``: a cell
    index below 1, or above n without wrapping.
    """
    T = rho.dtype.type
    n1, n2, n3 = rho.shape
    L = [T(v) for v in box_size]
    bmin = [T(v) for v in box_min]
    x = np.asarray(x, dtype=T).copy()
    y = np.asarray(y, dtype=T).copy()
    z = np.asarray(z, dtype=T).copy()
    w = np.asarray(w, dtype=T)
    if wrap:
        x = np.where((x - bmin[0]) > L[0], x - L[0], x).astype(T)
        y = np.where((y - bmin[0]) > L[0], y - L[0], y).astype(T)
        z = np.where((z - bmin[0]) > L[0], z - L[0], z).astype(T)
    gx = _grid_coord(x, bmin[0], L[0], n1, T)
    gy = _grid_coord(y, bmin[1], L[1], n2, T)
    gz = _grid_coord(z, bmin[2], L[2], n3, T)
    x0 = np.floor(gx).astype(np.int64)
    y0 = np.floor(gy).astype(np.int64)
    z0 = np.floor(gz).astype(np.int64)
    wx1 = (gx - x0.astype(T)).astype(T)
    wx0 = (T(1) - wx1).astype(T)
    wy1 = (gy - y0.astype(T)).astype(T)
    wy0 = (T(1) - wy1).astype(T)
    wz1 = (gz - z0.astype(T)).astype(T)
    wz0 = (T(1) - wz1).astype(T)
    x0 = np.where(x0 == n1 + 1, 1, x0)
    y0 = np.where(y0 == n2 + 1, 1, y0)
    z0 = np.where(z0 == n3 + 1, 1, z0)
    x1 = np.where((x0 == n1) & wrap, 1, x0 + 1)
    y1 = np.where((y0 == n2) & wrap, 1, y0 + 1)
    z1 = np.where((z0 == n3) & wrap, 1, z0 + 1)
    for lo, hi, n in ((x0, x1, n1), (y0, y1, n2), (z0, z1, n3)):
        if lo.size and (lo.min() < 1 or hi.max() > n):
            raise IndexError("paint index out of bounds (reference: BoundsError)")
    wx0 = wx0 * w
    wx1 = wx1 * w
    # the reference's corner order within one particle (src/mas.jl:42-49)
    corners = [
        (x0, y0, z0, wx0 * wy0 * wz0), (x1, y0, z0, wx1 * wy0 * wz0),
        (x0, y1, z0, wx0 * wy1 * wz0), (x0, y0, z1, wx0 * wy0 * wz1),
        (x1, y1, z0, wx1 * wy1 * wz0), (x1, y0, z1, wx1 * wy0 * wz1),
        (x0, y1, z1, wx0 * wy1 * wz1), (x1, y1, z1, wx1 * wy1 * wz1),
    ]
    idx = np.stack([(cx - 1) + n1 * ((cy - 1) + n2 * (cz - 1)) for cx, cy, cz, _ in corners], axis=1)
    val = np.stack([c[3].astype(T) for c in corners], axis=1)
    flat = rho.reshape(-1, order="F")
    # particle-major order: each cell receives its additions in particle order
    np.add.at(flat, idx.ravel(), val.ravel())
    rho[...] = flat.reshape(rho.shape, order="F")
    return rho, (x, y, z)


def cell_keys(x, y, z, box_size, box_min, dims, wrap=True):
    """0-based lower cell index ``(ix0, iy0, iz0)`` of every particle after the
    reference's wrap rules (``src/mas.jl:7-35``), and the linear key
    ``ix0 + n1·(iy0 + n2·iz0)``.  Integer output: compared bit-exactly."""
    T = np.float32
    n1, n2, n3 = dims
    L = [T(v) for v in box_size]
    bmin = [T(v) for v in box_min]
    x = np.asarray(x, dtype=T)
    y = np.asarray(y, dtype=T)
    z = np.asarray(z, dtype=T)
    if wrap:
        x = np.where((x - bmin[0]) > L[0], x - L[0], x).astype(T)
        y = np.where((y - bmin[0]) > L[0], y - L[0], y).astype(T)
        z = np.where((z - bmin[0]) > L[0], z - L[0], z).astype(T)
    out = []
    for p, a, n in ((x, 0, n1), (y, 1, n2), (z, 2, n3)):
        g = _grid_coord(p, bmin[a], L[a], n, T)
        i0 = np.floor(g).astype(np.int64)
        i0 = np.where(i0 == n + 1, 1, i0)
        out.append(i0 - 1)
    key = out[0] + n1 * (out[1] + n2 * out[2])
    return out[0], out[1], out[2], key


def cell_counts(x, y, z, box_size, box_min, dims, wrap=True):
    """Particle count per cell (by lower CIC cell), int64 mesh ``[ix,iy,iz]``."""
    *_, key = cell_keys(x, y, z, box_size, box_min, dims, wrap)
    n1, n2, n3 = dims
    c = np.bincount(key, minlength=n1 * n2 * n3)
    return c.reshape((n1, n2, n3), order="F")


def tsc(rho, x, y, z, w, box_size, box_min, wrap=True):
    """Triangular-shaped-cloud paint (no reference implementation).

    Same node convention as the reference CIC (node ``i`` at
    ``box_min + i·cell``, grid coordinate ``g = (p-box_min)·n/L``), periodic
    when ``wrap``: nearest node ``c = floor(g + 1/2)``, ``d = g - c``, weights
    ``0.5(0.5-d)²``, ``0.75-d²``, ``0.5(0.5+d)²`` on nodes ``c-1, c, c+1``.
    Positions are wrapped like the CIC paint does.
    """
    T = rho.dtype.type
    n = rho.shape
    L = [T(v) for v in box_size]
    bmin = [T(v) for v in box_min]
    P = [np.asarray(p, dtype=T).copy() for p in (x, y, z)]
    if wrap:
        P = [np.where((p - bmin[0]) > L[0], p - L[0], p).astype(T) for p in P]
    idx = []
    wts = []
    for a in range(3):
        g = (P[a] - bmin[a]) * T(n[a]) / L[a]
        c = np.floor(g + T(0.5)).astype(np.int64)
        d = (g - c.astype(T)).astype(T)
        wm = T(0.5) * (T(0.5) - d) * (T(0.5) - d)
        w0 = T(0.75) - d * d
        wp = T(0.5) * (T(0.5) + d) * (T(0.5) + d)
        ii = np.stack([c - 1, c, c + 1], axis=1)
        if wrap:
            ii = np.mod(ii, n[a])
        elif ii.size and (ii.min() < 0 or ii.max() >= n[a]):
            raise IndexError("TSC index out of bounds")
        idx.append(ii)
        wts.append(np.stack([wm, w0, wp], axis=1).astype(T))
    w = np.asarray(w, dtype=T)
    flat = rho.reshape(-1, order="F")
    cells = []
    vals = []
    for c in range(3):
        for b in range(3):
            for a in range(3):
                cells.append(idx[0][:, a] + n[0] * (idx[1][:, b] + n[1] * idx[2][:, c]))
                vals.append(((w * wts[0][:, a]) * wts[1][:, b]) * wts[2][:, c])
    np.add.at(flat, np.stack(cells, 1).ravel(), np.stack(vals, 1).astype(T).ravel())
    rho[...] = flat.reshape(rho.shape, order="F")
    return rho, tuple(P)


def read_cic(field, x, y, z, box_size, box_min, wrap=True):
    """Trilinear read-out, ``src/mas.jl:218-269`` (CPU method).

    ``cell = T(L/n)``; ``d = (p - box_min)/cell``; the eight products and the
    sum are evaluated left to right in T, so an FP32 result is bit-exact with
    the reference's arithmetic given the same mesh.
    """
    T = field.dtype.type
    n = field.shape
    out_idx = []
    fr = []
    for a, p in enumerate((x, y, z)):
        cell = T(T(box_size[a]) / T(n[a]))
        d = (np.asarray(p, dtype=T) - T(box_min[a])) / cell
        i = np.floor(d).astype(np.int64)
        u = (d - i.astype(T)).astype(T)
        dd = (T(1) - u).astype(T)
        i = i + 1
        lo = np.where((i > n[a]) & wrap, i - n[a], i)
        hi = lo + 1
        hi = np.where((hi > n[a]) & wrap, hi - n[a], hi)
        if lo.size and (lo.min() < 1 or hi.max() > n[a]):
            raise IndexError("read-out index out of bounds (reference: BoundsError)")
        out_idx.append((lo - 1, hi - 1))
        fr.append((dd, u))
    (xd, xu), (yd, yu), (zd, zu) = out_idx
    (dx, ux), (dy, uy), (dz, uz) = fr
    f = field
    terms = [
        f[xd, yd, zd] * dx * dy * dz, f[xd, yd, zu] * dx * dy * uz,
        f[xd, yu, zd] * dx * uy * dz, f[xd, yu, zu] * dx * uy * uz,
        f[xu, yd, zd] * ux * dy * dz, f[xu, yd, zu] * ux * dy * uz,
        f[xu, yu, zd] * ux * uy * dz, f[xu, yu, zu] * ux * uy * uz,
    ]
    acc = terms[0]
    for t in terms[1:]:
        acc = acc + t
    return acc.astype(T)


def fd_gradient_mesh(phi, box_size):
    """Periodic central-difference gradient mesh of the finite-difference
    read-out: component a is ``(φ[c + e_a] - φ[c - e_a]) / cell2_a`` with
    ``cell2_a = T(2 L_a) / n_a`` as ``src/mas.jl:390`` spells the doubled cell
    (``cell = 2 * box_size / dims``); evaluated in T, so an FP32 mesh is
    bit-exact with the device's."""
    T = phi.dtype.type
    out = []
    for a in range(3):
        c2 = T(T(T(2) * T(box_size[a])) / T(phi.shape[a]))
        diff = (np.roll(phi, -1, axis=a) - np.roll(phi, 1, axis=a)).astype(T)
        out.append((diff / c2).astype(T))
    return tuple(out)


def read_grad_cic(field, x, y, z, box_size, box_min):
    """The finite-difference read-out ``read_grad_cic`` of ``src/mas.jl:388-466``
    (commented out in the reference; pyrecon's finite-difference read-out) in
    FP64: for each particle, the CIC-weighted sum over its 8 surrounding nodes
    of the node's central differences ``φ[n + e_a] - φ[n - e_a]`` (periodic),
    divided by ``2 L_a / n_a``.  The particle's grid coordinate uses the cell
    ``L / n``: the commented-out code divides the position by the doubled cell
    as well, which places a particle at half its grid coordinate; pyrecon and
    this restatement do not."""
    f = np.asarray(field, dtype=np.float64)
    n = f.shape
    base, frac = [], []
    for a, p in enumerate((x, y, z)):
        d = (np.asarray(p, dtype=np.float64) - float(box_min[a])) / (float(box_size[a]) / n[a])
        i = np.floor(d).astype(np.int64)
        base.append(i)
        frac.append(d - i)
    out = [np.zeros(len(base[0])) for _ in range(3)]
    for cx in (0, 1):
        for cy in (0, 1):
            for cz in (0, 1):
                w = ((frac[0] if cx else 1 - frac[0]) * (frac[1] if cy else 1 - frac[1])
                     * (frac[2] if cz else 1 - frac[2]))
                node = [(base[0] + cx) % n[0], (base[1] + cy) % n[1], (base[2] + cz) % n[2]]
                for a in range(3):
                    up = list(node)
                    dn = list(node)
                    up[a] = (node[a] + 1) % n[a]
                    dn[a] = (node[a] - 1) % n[a]
                    out[a] += w * (f[tuple(up)] - f[tuple(dn)])
    return tuple(out[a] / (2.0 * float(box_size[a]) / n[a]) for a in range(3))


# ----------------------------------------------------------------------------
# Overdensity — src/recon.jl:42-91
# ----------------------------------------------------------------------------

def setup_overdensity(delta, bias, R, box_size, box_min, x, y, z, w, wrap=True,
                      mas="cic"):
    """Data-only overdensity, ``src/recon.jl:42-57``: paint (wrapping), smooth,
    ``δ = (δ/mean(δ) - 1)/b``.  Returns ``(δ, wrapped positions)``."""
    T = delta.dtype.type
    paint = cic if mas == "cic" else tsc
    delta, pos = paint(delta, x, y, z, w, box_size, box_min, wrap=wrap)
    delta = smooth(delta, R, box_size)
    mean = T(np.mean(delta, dtype=np.float64))
    delta = ((delta / mean - T(1)) / T(bias)).astype(T)
    return delta, pos


def setup_overdensity_randoms(delta, bias, R, box_size, box_min, x, y, z, w,
                              rx, ry, rz, rw, ran_min=0.01, mas="cic"):
    """Data + randoms overdensity, ``src/recon.jl:60-91``.

    Both catalogs are painted without wrapping and smoothed;
    ``α = Σδ_d/Σδ_r``; ``threshold = ran_min·Σδ_r/N_rand`` (count, not weight
    sum); ``δ = δ_r > thr ? (δ_d - αδ_r)/(b α δ_r) : 0``.
    """
    T = delta.dtype.type
    paint = cic if mas == "cic" else tsc
    ran = np.zeros_like(delta)
    delta, _ = paint(delta, x, y, z, w, box_size, box_min, wrap=False)
    ran, _ = paint(ran, rx, ry, rz, rw, box_size, box_min, wrap=False)
    delta = smooth(delta, R, box_size)
    ran = smooth(ran, R, box_size)
    sd = np.sum(delta, dtype=np.float64)
    sr = np.sum(ran, dtype=np.float64)
    alpha = T(sd / sr)
    thr = T(T(ran_min) * T(sr) / T(len(rx)))
    delta = (delta - alpha * ran).astype(T)
    denom = (T(bias) * alpha * ran).astype(T)
    safe = np.where(ran > thr, denom, T(1))
    delta = np.where(ran > thr, delta / safe, T(0)).astype(T)
    return delta


# ----------------------------------------------------------------------------
# Iterative FFT reconstruction — src/iterative.jl
# ----------------------------------------------------------------------------

def iterate(delta_r, delta_s, k, it, beta, los=None, xv=None):
    """One iteration, ``src/iterative.jl:5-67`` (CPU method).

    ``δ_k = rfft(δ_r)/k²`` (k=0 → 0); ``δ_r := δ_s``; then for local LOS and
    every ``i ≤ j``: ``δ_r -= fac · irfft(k_i k_j δ_k) · x_i x_j / x²`` with
    ``fac = (1+[i≠j])β`` (divided by ``1+β`` on iteration 1) and δ_r set to 0
    where ``x² = 0``; for a global LOS ``r̂`` and every axis with
    ``r̂_i ≠ 0``: ``δ_r -= fac · irfft(k_i² r̂_i δ_k)``.
    """
    T = delta_r.dtype.type
    beta = T(beta)
    n1 = delta_r.shape[0]
    dk = rfft3(delta_r)
    k2 = _k2(k, T)
    k2 = np.where(k2 == 0, T(1), k2)
    dk = dk / k2
    dk[0, 0, 0] = 0
    out = delta_s.copy()
    kk = _kk(k, None)
    if los is None:
        assert xv is not None
        X = (xv[0][:, None, None], xv[1][None, :, None], xv[2][None, None, :])
        x2 = (X[0] * X[0] + X[1] * X[1]) + X[2] * X[2]
        for i in range(3):
            for j in range(i, 3):
                fac = T((T(1) + T(i != j)) * beta)
                if it == 1:
                    fac = T(fac / (T(1) + beta))
                dij = irfft3((kk[i] * kk[j]) * dk, n1).astype(T)
                upd = out - fac * dij * X[i] * X[j] / np.where(x2 > 0, x2, T(1))
                out = np.where(x2 > 0, upd, T(0)).astype(T)
    else:
        r = [T(v) for v in los]
        for i in range(3):
            if r[i] == 0:
                continue
            fac = beta
            if it == 1:
                fac = T(fac / (T(1) + beta))
            di = irfft3((kk[i] * kk[i] * r[i]) * dk, n1).astype(T)
            out = (out - fac * di).astype(T)
    return out


def reconstructed_overdensity(delta, bias, f, R, box_size, box_min, n_iter,
                              x, y, z, w, los=None, randoms=None, mas="cic"):
    """``src/recon.jl:93-132``: overdensity, ``δ_s = copy(δ)``, then
    ``n_iter`` calls of :func:`iterate` with the 1-based iteration counter.
    Returns ``(δ_r, wrapped data positions or None)``."""
    T = delta.dtype.type
    beta = T(T(f) / T(bias))
    pos = None
    if randoms is None:
        delta, pos = setup_overdensity(delta, bias, R, box_size, box_min, x, y, z, w, mas=mas)
    else:
        delta = setup_overdensity_randoms(delta, bias, R, box_size, box_min, x, y, z, w,
                                          *randoms, mas=mas)
    ds = delta.copy()
    k = k_vec(delta.shape, box_size, T)
    xv = x_vec(delta.shape, box_size, box_min, T) if los is None else None
    for it in range(1, n_iter + 1):
        delta = iterate(delta, ds, k, it, beta, los=los, xv=xv)
    return delta, pos


def compute_displacements_iterative(delta_r, x, y, z, box_size, box_min):
    """``src/iterative.jl:253-275``: ``Ψ_i = irfft(i k_i δ_k / k²)`` (k=0 → 0),
    read at the particles with :func:`read_cic`."""
    T = delta_r.dtype.type
    n1 = delta_r.shape[0]
    k = k_vec(delta_r.shape, box_size, T)
    dk = rfft3(delta_r)
    k2 = _k2(k, T)
    kk = _kk(k, None)
    out = []
    for i in range(3):
        psik = np.where(k2 > 0, (1j * kk[i]) * dk / np.where(k2 > 0, k2, T(1)), 0).astype(dk.dtype)
        psik[0, 0, 0] = 0
        psir = irfft3(psik, n1).astype(T)
        out.append(read_cic(psir, x, y, z, box_size, box_min))
    return tuple(out)


def displacement_meshes_iterative(delta_r, box_size):
    """The three Ψ meshes of :func:`compute_displacements_iterative`."""
    T = delta_r.dtype.type
    n1 = delta_r.shape[0]
    k = k_vec(delta_r.shape, box_size, T)
    dk = rfft3(delta_r)
    k2 = _k2(k, T)
    kk = _kk(k, None)
    out = []
    for i in range(3):
        psik = np.where(k2 > 0, (1j * kk[i]) * dk / np.where(k2 > 0, k2, T(1)), 0).astype(dk.dtype)
        psik[0, 0, 0] = 0
        out.append(irfft3(psik, n1).astype(T))
    return tuple(out)


def gradient_meshes(phi, box_size):
    """``∂_i φ = irfft(i k_i φ_k)``, ``src/multigrid.jl:755-773``."""
    T = phi.dtype.type
    n1 = phi.shape[0]
    k = k_vec(phi.shape, box_size, T)
    pk = rfft3(phi)
    kk = _kk(k, None)
    return tuple(irfft3(((1j * kk[i]) * pk).astype(pk.dtype), n1).astype(T) for i in range(3))


def compute_displacements_multigrid(phi, x, y, z, box_size, box_min):
    """``src/multigrid.jl:755-773``: spectral gradient of φ read at the particles."""
    return tuple(read_cic(g, x, y, z, box_size, box_min) for g in gradient_meshes(phi, box_size))


def read_shifts(disp, x, y, z, f, los=None, field="disp"):
    """``src/recon.jl:264-306``: ``:disp`` → Ψ; ``:rsd`` → ``f(Ψ·r̂)r̂`` with
    ``r̂ = p/|p|`` (local) or the given LOS; ``:sum`` → Ψ + rsd."""
    T = disp[0].dtype.type
    f = T(f)
    if field == "disp":
        return tuple(d.copy() for d in disp)
    x = np.asarray(x, dtype=T)
    y = np.asarray(y, dtype=T)
    z = np.asarray(z, dtype=T)
    if los is None:
        dist = np.sqrt(x * x + y * y + z * z)
        lx, ly, lz = x / dist, y / dist, z / dist
        dot = (disp[0] * lx + disp[1] * ly) + disp[2] * lz
        rsd = (f * dot * lx, f * dot * ly, f * dot * lz)
    else:
        l = [T(v) for v in los]
        dot = (disp[0] * l[0] + disp[1] * l[1]) + disp[2] * l[2]
        rsd = tuple(f * dot * l[j] for j in range(3))
    rsd = tuple(r.astype(T) for r in rsd)
    if field == "rsd":
        return rsd
    if field == "sum":
        return tuple((disp[j] + rsd[j]).astype(T) for j in range(3))
    raise ValueError(f"unknown field {field!r}")


def reconstructed_positions(shifts, x, y, z):
    """``src/recon.jl:366-380``: ``p_rec = p - shift``."""
    T = shifts[0].dtype.type
    return tuple((np.asarray(p, dtype=T) - s).astype(T) for p, s in zip((x, y, z), shifts))


# ----------------------------------------------------------------------------
# Multigrid — src/multigrid.jl
# ----------------------------------------------------------------------------

def stencil_coefficients(dims, box_size, box_min, beta, los=None, dtype=np.float32):
    """Per-cell coefficients of the anisotropic operator (``src/multigrid.jl:17-29,
    55-62``): ``p = x_vec/cell`` (local) or ``los/cell`` (global);
    ``g = β/Σ cell_i² p_i²``; ``gp_i = 1/cell_i² + g p_i²``.  Returns
    broadcastable ``(px, py, pz, g, gpx2, gpy2, gpz2)``."""
    T = dtype
    n = dims
    cell = [T(T(box_size[a]) / T(n[a])) for a in range(3)]
    cell2 = [T(c * c) for c in cell]
    icell2 = [T(T(1) / c2) for c2 in cell2]
    beta = T(beta)
    if los is None:
        xv = x_vec(dims, box_size, box_min, T)
        px = (xv[0] / cell[0])[:, None, None]
        py = (xv[1] / cell[1])[None, :, None]
        pz = (xv[2] / cell[2])[None, None, :]
    else:
        px = np.array(T(T(los[0]) / cell[0]), dtype=T).reshape(1, 1, 1)
        py = np.array(T(T(los[1]) / cell[1]), dtype=T).reshape(1, 1, 1)
        pz = np.array(T(T(los[2]) / cell[2]), dtype=T).reshape(1, 1, 1)
    # Julia evaluates c2 * p^2 and g * p^2 with the power first
    g = beta / ((cell2[0] * (px * px) + cell2[1] * (py * py)) + cell2[2] * (pz * pz))
    gpx2 = icell2[0] + g * (px * px)
    gpy2 = icell2[1] + g * (py * py)
    gpz2 = icell2[2] + g * (pz * pz)
    return px, py, pz, g, gpx2, gpy2, gpz2


def _nb(v):
    """Periodic neighbour views of v: dict offset → shifted array."""
    out = {}
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                if abs(dx) + abs(dy) + abs(dz) in (1, 2):
                    out[(dx, dy, dz)] = np.roll(v, shift=(-dx, -dy, -dz), axis=(0, 1, 2))
    return out


def _offdiag(v, coef, local):
    """Neighbour part of the stencil, ``src/multigrid.jl:64-79`` (the bracket
    added to f in ``jac``)."""
    px, py, pz, g, gpx2, gpy2, gpz2 = coef
    T = v.dtype.type
    N = _nb(v)
    s = (gpx2 * (N[(1, 0, 0)] + N[(-1, 0, 0)]) + gpy2 * (N[(0, 1, 0)] + N[(0, -1, 0)])
         + gpz2 * (N[(0, 0, 1)] + N[(0, 0, -1)])
         + g / T(2) * (px * py * (N[(1, 1, 0)] + N[(-1, -1, 0)] - N[(-1, 1, 0)] - N[(1, -1, 0)])
                       + px * pz * (N[(1, 0, 1)] + N[(-1, 0, -1)] - N[(-1, 0, 1)] - N[(1, 0, -1)])
                       + py * pz * (N[(0, 1, 1)] + N[(0, -1, -1)] - N[(0, -1, 1)] - N[(0, 1, -1)])))
    if local:
        s = s + g * (px * (N[(1, 0, 0)] - N[(-1, 0, 0)]) + py * (N[(0, 1, 0)] - N[(0, -1, 0)])
                     + pz * (N[(0, 0, 1)] - N[(0, 0, -1)]))
    return s


def apply_operator(v, coef, local):
    """``A v`` with ``A v = 2Σgp_i v - (neighbour part)`` so that the residual
    is ``f - A v`` (``src/multigrid.jl:262-276``)."""
    px, py, pz, g, gpx2, gpy2, gpz2 = coef
    T = v.dtype.type
    return (T(2) * (gpx2 + gpy2 + gpz2) * v - _offdiag(v, coef, local)).astype(T)


def jacobi(v, f, box_size, box_min, beta, damping, niter, los=None):
    """Damped Jacobi, ``src/multigrid.jl:14-135``:
    ``jac = (f + neighbours)/(2Σgp)``; ``v = (1-ω)v + ω·jac``, ``niter`` times."""
    T = v.dtype.type
    coef = stencil_coefficients(v.shape, box_size, box_min, beta, los, T)
    diag = T(2) * (coef[4] + coef[5] + coef[6])
    om = T(damping)
    for _ in range(niter):
        jac = (f + _offdiag(v, coef, los is None)) / diag
        v = ((T(1) - om) * v + om * jac).astype(T)
    return v


def residual(v, f, box_size, box_min, beta, los=None):
    """``r = f - A v``, ``src/multigrid.jl:213-326``."""
    T = v.dtype.type
    coef = stencil_coefficients(v.shape, box_size, box_min, beta, los, T)
    return (f - apply_operator(v, coef, los is None)).astype(T)


def prolong(v2h, fine_shape):
    """Trilinear prolongation, ``src/multigrid.jl:398-453``.  Coarse node ``c``
    (0-based) lands on fine node ``2c+1``; fine ``2c+2`` averages ``c, c+1``
    (periodic).  The target is overwritten."""
    T = v2h.dtype.type
    v1h = np.zeros(fine_shape, dtype=T)
    c = v2h
    cx = np.roll(c, -1, 0)
    cy = np.roll(c, -1, 1)
    cz = np.roll(c, -1, 2)
    cxy = np.roll(cx, -1, 1)
    cxz = np.roll(cx, -1, 2)
    cyz = np.roll(cy, -1, 2)
    cxyz = np.roll(cxy, -1, 2)
    o = slice(1, None, 2)   # fine 2c+1
    e = slice(2, None, 2)   # fine 2c+2 for c < n-1; index 0 holds c = n-1

    def put(sx, sy, sz, val):
        # fine index 2c+2 wraps to 0 for the last coarse node
        fx = np.r_[1:fine_shape[0]:2] if sx == 0 else (np.arange(c.shape[0]) * 2 + 2) % fine_shape[0]
        fy = np.r_[1:fine_shape[1]:2] if sy == 0 else (np.arange(c.shape[1]) * 2 + 2) % fine_shape[1]
        fz = np.r_[1:fine_shape[2]:2] if sz == 0 else (np.arange(c.shape[2]) * 2 + 2) % fine_shape[2]
        v1h[np.ix_(fx, fy, fz)] = val

    put(0, 0, 0, c)
    put(1, 0, 0, (c + cx) / T(2))
    put(0, 1, 0, (c + cy) / T(2))
    put(0, 0, 1, (c + cz) / T(2))
    put(1, 1, 0, (c + cx + cy + cxy) / T(4))
    put(0, 1, 1, (c + cy + cz + cyz) / T(4))
    put(1, 0, 1, (c + cx + cz + cxz) / T(4))
    put(1, 1, 1, (c + cx + cy + cz + cxy + cxz + cyz + cxyz) / T(8))
    del o, e
    return v1h


def reduce(v1h):
    """Full-weighting restriction, ``src/multigrid.jl:520-584``: coarse ``c``
    is centred on fine ``2c+1``, weights 8/4/2/1 over 64, periodic."""
    T = v1h.dtype.type
    N = {}
    for dx in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dz in (-1, 0, 1):
                N[(dx, dy, dz)] = np.roll(v1h, shift=(-dx, -dy, -dz), axis=(0, 1, 2))[1::2, 1::2, 1::2]
    faces = [k for k in N if sum(map(abs, k)) == 1]
    edges = [k for k in N if sum(map(abs, k)) == 2]
    corners = [k for k in N if sum(map(abs, k)) == 3]
    s = T(8) * N[(0, 0, 0)] + T(4) * sum(N[k] for k in faces) + T(2) * sum(N[k] for k in edges) \
        + sum(N[k] for k in corners)
    return (s / T(64)).astype(T)


def _can_recurse(shape):
    return all(n > 4 and n % 2 == 0 for n in shape)


def vcycle(v, f, box_size, box_min, beta, damping, niter, los=None):
    """V-cycle, ``src/multigrid.jl:654-687``: pre-smooth, residual, restrict,
    recursive V-cycle from zero, prolong, correct, post-smooth."""
    T = v.dtype.type
    v = jacobi(v, f, box_size, box_min, beta, damping, niter, los)
    if _can_recurse(v.shape):
        r = residual(v, f, box_size, box_min, beta, los)
        f2h = reduce(r)
        v2h = vcycle(np.zeros_like(f2h), f2h, box_size, box_min, beta, damping, niter, los)
        v = (v + prolong(v2h, v.shape)).astype(T)
    return jacobi(v, f, box_size, box_min, beta, damping, niter, los)


def fmg(f1h, box_size, box_min, beta, damping, niter, ncycles, los=None):
    """Full multigrid, ``src/multigrid.jl:722-752``: restrict f to the coarsest
    level, then on the way up prolong the coarse solution (overwriting any
    guess) and run ``ncycles`` V-cycles.  No residual test."""
    if _can_recurse(f1h.shape):
        v2h = fmg(reduce(f1h), box_size, box_min, beta, damping, niter, ncycles, los)
        v1h = prolong(v2h, f1h.shape)
    else:
        v1h = np.zeros_like(f1h)
    for _ in range(ncycles):
        v1h = vcycle(v1h, f1h, box_size, box_min, beta, damping, niter, los)
    return v1h


def reconstructed_potential(phi_shape, bias, f, R, box_size, box_min, x, y, z, w,
                            randoms=None, los=None, damping=0.4, niter=5, ncycles=6,
                            dtype=np.float32, mas="cic"):
    """``src/recon.jl:184-212``: overdensity, then :func:`fmg` with rhs δ."""
    T = dtype
    beta = T(T(f) / T(bias))
    delta = np.zeros(phi_shape, dtype=T)
    if randoms is None:
        delta, _ = setup_overdensity(delta, bias, R, box_size, box_min, x, y, z, w, mas=mas)
    else:
        delta = setup_overdensity_randoms(delta, bias, R, box_size, box_min, x, y, z, w,
                                          *randoms, mas=mas)
    return fmg(delta, box_size, box_min, beta, T(damping), niter, ncycles, los), delta


def run_iterative(grid, bias, f, R, x, y, z, w, box_size=None, box_min=None, los=None,
                  n_iter=3, randoms=None, dtype=np.float32, mas="cic"):
    """``run!(::IterativeRecon, ...)``, ``src/recon.jl:134-180``.  With randoms
    the box is replaced by ``setup_box(randoms, 500)``.  Returns
    ``(δ_r, box_size, box_min, wrapped data positions or None)``."""
    T = dtype
    if randoms is not None:
        box_size, box_min = setup_box(randoms[0], randoms[1], randoms[2], 500, T)
    delta = np.zeros(grid, dtype=T)
    delta, pos = reconstructed_overdensity(delta, bias, f, R, box_size, box_min, n_iter,
                                           x, y, z, w, los=los, randoms=randoms, mas=mas)
    return delta, box_size, box_min, pos


def run_multigrid(grid, bias, f, R, x, y, z, w, box_size=None, box_min=None, los=None,
                  damping=0.4, niter=5, ncycles=6, randoms=None, dtype=np.float32, mas="cic"):
    """``run!(::MultigridRecon, ...)``, ``src/recon.jl:215-261``."""
    T = dtype
    if randoms is not None:
        box_size, box_min = setup_box(randoms[0], randoms[1], randoms[2], 500, T)
    phi, _ = reconstructed_potential(grid, bias, f, R, box_size, box_min, x, y, z, w,
                                     randoms=randoms, los=los, damping=damping, niter=niter,
                                     ncycles=ncycles, dtype=T, mas=mas)
    return phi, box_size, box_min


# ----------------------------------------------------------------------------
# Convergent multigrid (no reference implementation): own oracle
# ----------------------------------------------------------------------------

def clamp_coefficients(coef, kappa):
    """Coefficients with the first-derivative term limited to
    ``|g p_a| <= κ gp_a`` (the V-cycle operator of the convergent solver; only
    cells next to the observer change)."""
    px, py, pz, g, gpx2, gpy2, gpz2 = coef
    d = [g * px, g * py, g * pz]
    gp = [gpx2, gpy2, gpz2]
    d = [np.clip(d[a], -kappa * gp[a], kappa * gp[a]) for a in range(3)]
    return (px, py, pz, g, gpx2, gpy2, gpz2, d[0], d[1], d[2])


def _offdiag_any(v, coef, local):
    if len(coef) == 7:
        return _offdiag(v, coef, local)
    px, py, pz, g, gpx2, gpy2, gpz2, dx, dy, dz = coef
    T = v.dtype.type
    N = _nb(v)
    s = (gpx2 * (N[(1, 0, 0)] + N[(-1, 0, 0)]) + gpy2 * (N[(0, 1, 0)] + N[(0, -1, 0)])
         + gpz2 * (N[(0, 0, 1)] + N[(0, 0, -1)])
         + g / T(2) * (px * py * (N[(1, 1, 0)] + N[(-1, -1, 0)] - N[(-1, 1, 0)] - N[(1, -1, 0)])
                       + px * pz * (N[(1, 0, 1)] + N[(-1, 0, -1)] - N[(-1, 0, 1)] - N[(1, 0, -1)])
                       + py * pz * (N[(0, 1, 1)] + N[(0, -1, -1)] - N[(0, -1, 1)] - N[(0, 1, -1)])))
    if local:
        s = s + (dx * (N[(1, 0, 0)] - N[(-1, 0, 0)]) + dy * (N[(0, 1, 0)] - N[(0, -1, 0)])
                 + dz * (N[(0, 0, 1)] - N[(0, 0, -1)]))
    return s


def gauss_seidel_rb(v, f, coef, local, nsweeps):
    """Red-black Gauss-Seidel sweeps on ``A v = f`` (colour = (i+j+k) mod 2,
    red first).  For the 19-point operator the edge neighbours share a colour,
    so a colour update reads their pre-sweep values (hybrid ordering)."""
    T = v.dtype.type
    diag = T(2) * (coef[4] + coef[5] + coef[6])
    n1, n2, n3 = v.shape
    ii = np.add.outer(np.add.outer(np.arange(n1), np.arange(n2)), np.arange(n3)) % 2
    for _ in range(nsweeps):
        for colour in (0, 1):
            upd = (f + _offdiag_any(v, coef, local)) / diag
            v = np.where(ii == colour, upd, v).astype(T)
    return v


def _coarse_solve(f, coef, local, sweeps):
    """Coarsest level: mean-free right-hand side, red-black sweeps, mean-free result."""
    f = f - f.mean()
    v = gauss_seidel_rb(np.zeros_like(f), f, coef, local, sweeps)
    return v - v.mean()


def solve_mg(f, box_size, box_min, beta, los=None, rtol=1e-6, max_cycles=50, nu1=2, nu2=2, v0=None,
             coarse_sweeps=200, kappa=0.5):
    """Residual-driven multigrid (own method, no reference counterpart).

    The periodic operator annihilates constants and, for the local line of
    sight, its left null vector is not constant, so ``A v = f`` is solvable
    only after shifting ``f`` by a constant ``α``.  Defect correction finds
    both::

        r_k = f - α_k - A v_k;  α_{k+1} = α_k + mean(r_k);
        v_{k+1} = v_k + V(r_k - mean(r_k))

    where ``V`` is one V-cycle (``nu1``/``nu2`` red-black sweeps, full-weighting
    restriction and trilinear prolongation of the reference, clamped
    first-derivative coefficients, ``coarse_sweeps`` sweeps on the coarsest
    level).  Stops when ``|r_k| <= rtol |f - α_k|``.  Returns
    ``(v, history, α)``.
    """
    T = f.dtype.type
    local = los is None
    levels = [f.shape]
    while _can_recurse(levels[-1]):
        levels.append(tuple(n // 2 for n in levels[-1]))
    exact = stencil_coefficients(f.shape, box_size, box_min, beta, los, T)
    pre = [clamp_coefficients(stencil_coefficients(s, box_size, box_min, beta, los, T), T(kappa))
           for s in levels]

    def A_pre(v, l):
        c = pre[l]
        return (T(2) * (c[4] + c[5] + c[6]) * v - _offdiag_any(v, c, local)).astype(T)

    def cycle(rhs, l):
        if l == len(levels) - 1:
            return _coarse_solve(rhs, pre[l], local, coarse_sweeps)
        e = gauss_seidel_rb(np.zeros_like(rhs), rhs, pre[l], local, nu1)
        r = (rhs - A_pre(e, l)).astype(T)
        e = (e + prolong(cycle(reduce(r), l + 1), e.shape)).astype(T)
        return gauss_seidel_rb(e, rhs, pre[l], local, nu2)

    v = np.zeros_like(f) if v0 is None else v0.astype(T).copy()
    alpha = float(np.mean(f, dtype=np.float64))
    hist = []
    for k in range(max_cycles + 1):
        r = (f - T(alpha) - apply_operator(v, exact, local)).astype(T)
        fn = float(np.linalg.norm((f - T(alpha)).astype(np.float64)))
        hist.append(float(np.linalg.norm(r.astype(np.float64))) / fn)
        if hist[-1] <= rtol or k == max_cycles:
            break
        m = float(np.mean(r, dtype=np.float64))
        alpha += m
        v = (v + cycle((r - T(m)).astype(T), 0)).astype(T)
    return v, hist, alpha


def coefs_f64(c):
    """Coefficient arrays promoted to FP64 (same values)."""
    return tuple(np.asarray(a, dtype=np.float64) for a in c)


# ---- catalog coordinates (examples/lightcone.jl:30-82) ------------------------

def _interp_uniform(zg, r, z):
    """Gridded(Linear()) interpolation of r on the uniform grid zg (src/cosmo.jl:83-90)."""
    return np.interp(np.asarray(z, np.float64), zg, r)


def sky_to_cartesian(ra, dec, red, zg, r, h):
    """examples/lightcone.jl:30-47: FP32 angles (x * Float32(π) / 180), FP32
    trigonometry, FP64 distance products stored as FP32."""
    F = np.float32
    pi = F(np.pi)
    a = (np.asarray(ra, F) * pi) / F(180)
    d = (np.asarray(dec, F) * pi) / F(180)
    dist = _interp_uniform(zg, r, red)
    cd, sd, ca, sa = (np.cos(d).astype(np.float64), np.sin(d).astype(np.float64),
                      np.cos(a).astype(np.float64), np.sin(a).astype(np.float64))
    hh = float(F(h))
    return ((dist * cd * ca * hh).astype(F), (dist * cd * sa * hh).astype(F), (dist * sd * hh).astype(F))


def cartesian_to_sky(x, y, z, zg, r, h):
    """examples/lightcone.jl:50-80, including ra = (lon - 360) rem 360."""
    F = np.float32
    x, y, z = (np.asarray(v, F) for v in (x, y, z))
    rr = np.sqrt(x * x + y * y + z * z) / F(h)
    s = np.sqrt(x * x + y * y)
    lon = (np.arctan2(y, x) * F(180)) / F(np.pi)
    lat = (np.arctan2(z, s) * F(180)) / F(np.pi)
    lon = np.fmod(lon - F(360), F(360))
    red = np.interp(rr.astype(np.float64), r, zg)
    return lon.astype(F), lat.astype(F), red.astype(F)


def fkp_weights(nz, P0):
    """examples/lightcone.jl:82."""
    F = np.float32
    return (F(1) / (F(1) + np.asarray(nz, F) * F(P0))).astype(F)
