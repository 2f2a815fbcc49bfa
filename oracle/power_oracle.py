"""CPU oracle of the power-spectrum multipoles (test infrastructure: only the
tests import it).

The reference checks its reconstructions with the external pypowspec
(``compute_auto_box``, ``compute_auto_box_rand``, ``compute_auto_lc``
called from ``test_helpers/simulation.py:40-55`` and
``test_helpers/lightcone.py:48-75``), which is not part of the reference
tree.  This module restates the published estimators those functions
implement, in FP64 NumPy with the full complex FFT:

* periodic box, fixed line of sight ``l``:
  ``P(k, mu) = |F_k / W(k)|^2 / I - shot``, ``mu = k.l / |k|``,
  ``P_ell = (2 ell + 1) <P(k, mu) L_ell(mu)>`` over the modes of a shell
  (shot noise only in ``P_0``);
* survey, local line of sight from the origin (Yamamoto estimator in the FFT
  form of Bianchi et al. 2015 / Scoccimarro 2015): ``A_0 = FFT[F]``,
  ``A_2 = sum_ij khat_i khat_j FFT[rhat_i rhat_j F]``,
  ``A_4 = sum_ijkl khat_i khat_j khat_k khat_l FFT[rhat_i rhat_j rhat_k rhat_l F]``
  with ``rhat`` at the mesh nodes; ``P_0 = <|A_0|^2>/I - shot``,
  ``P_2 = 5/2 <Re A_0 (3 A_2 - A_0)*>/I``,
  ``P_4 = 9/8 <Re A_0 (35 A_4 - 30 A_2 + 3 A_0)*>/I``.

Conventions shared with the device code: mesh nodes at ``box_min + i L/n``;
CIC or TSC weights, periodic; ``F = sum w_d - alpha sum w_r`` with
``alpha = sum w_d / sum w_r``; window ``W = prod_a sinc(k_a cell_a / 2)^p``
(``p`` = 2 CIC, 3 TSC); interlacing averages ``F_k`` with the transform of a
second paint shifted by half a cell, phase ``exp(i k.h)``; normalisation
``I = (sum w_d)^2 / V`` (box) or ``alpha sum_r n(z) w_r^2`` (survey);
``shot = (sum w_d^2 + alpha^2 sum w_r^2) / I``.  Parity with pypowspec
itself is unpinned: it is absent here and its default assignment and
interlacing choices are not visible from its call sites.
"""
from __future__ import annotations

import itertools
import math

import numpy as np


def paint(n, box_size, box_min, x, y, z, w, mas="cic", shift=0.0):
    """Periodic CIC/TSC paint of weights at grid coordinates
    ``(p - box_min) n / L + shift``; mesh indexed [ix, iy, iz]."""
    n = tuple(int(v) for v in n)
    mesh = np.zeros(n)
    w = np.ones(len(x)) if w is None else np.asarray(w, np.float64)
    idx, wts = [], []
    for a, p in enumerate((x, y, z)):
        u = (np.asarray(p, np.float64) - box_min[a]) * n[a] / box_size[a] + shift
        if mas == "tsc":
            c = np.floor(u + 0.5)
            d = u - c
            ci = c.astype(np.int64)
            idx.append([(ci - 1) % n[a], ci % n[a], (ci + 1) % n[a]])
            wts.append([0.5 * (0.5 - d) ** 2, 0.75 - d * d, 0.5 * (0.5 + d) ** 2])
        else:
            c = np.floor(u)
            f = u - c
            ci = c.astype(np.int64)
            idx.append([ci % n[a], (ci + 1) % n[a]])
            wts.append([1.0 - f, f])
    K = len(idx[0])
    for a, b, c in itertools.product(range(K), repeat=3):
        np.add.at(mesh, (idx[0][a], idx[1][b], idx[2][c]), w * wts[0][a] * wts[1][b] * wts[2][c])
    return mesh


def _kgrid(n, box_size):
    ks = [2 * np.pi * np.fft.fftfreq(n[a], d=box_size[a] / n[a]) for a in range(3)]
    return np.meshgrid(*ks, indexing="ij")


def _window(K, n, box_size, p):
    W = np.ones_like(K[0])
    for a in range(3):
        h = 0.5 * K[a] * box_size[a] / n[a]
        W = W * np.where(np.abs(h) < 1e-8, 1.0, np.sin(h) / np.where(h == 0, 1.0, h))
    return W ** p


def multipoles(geometry, n, box_size, box_min, data, randoms=None, rnz=None, mas="cic", interlace=False,
               los=(0.0, 0.0, 1.0), kmin=0.0, dk=0.01, nbins=10):
    """(k_mean, P0, P2, P4, nmodes, shot, norm); data = (x, y, z, w) with w
    possibly None, randoms likewise; geometry "box" or "survey"."""
    n = tuple(int(v) for v in n)
    L = [float(v) for v in box_size]
    bm = [float(v) for v in box_min]
    x, y, z, w = data
    wd = np.ones(len(x)) if w is None else np.asarray(w, np.float64)
    sd = (wd.sum(), (wd * wd).sum())
    if randoms is not None:
        rx, ry, rz, rw = randoms
        wr = np.ones(len(rx)) if rw is None else np.asarray(rw, np.float64)
        alpha = sd[0] / wr.sum()
        sr2 = (wr * wr).sum()
    else:
        alpha, sr2 = 0.0, 0.0
    V = L[0] * L[1] * L[2]
    if geometry == "survey":
        norm = alpha * float((np.asarray(rnz, np.float64) * wr * wr).sum())
    else:
        norm = sd[0] ** 2 / V
    shot = (sd[1] + alpha * alpha * sr2) / norm

    def field(shift):
        F = paint(n, L, bm, x, y, z, wd, mas, shift)
        if randoms is not None:
            F = F - alpha * paint(n, L, bm, rx, ry, rz, wr, mas, shift)
        return F

    F = field(0.0)
    A0 = np.fft.fftn(F)
    K = _kgrid(n, L)
    kk = np.sqrt(K[0] ** 2 + K[1] ** 2 + K[2] ** 2)
    if geometry == "box" and interlace:
        F2 = field(0.5)
        ph = 0.5 * sum(K[a] * L[a] / n[a] for a in range(3))
        A0 = 0.5 * (A0 + np.fft.fftn(F2) * np.exp(1j * ph))
    Wk = _window(K, n, L, 3 if mas == "tsc" else 2)
    inv = np.where(kk > 0, 1.0 / np.where(kk > 0, kk, 1.0), 0.0)
    khat = [K[a] * inv for a in range(3)]
    if geometry == "survey":
        g = [bm[a] + np.arange(n[a]) * L[a] / n[a] for a in range(3)]
        P = np.meshgrid(*g, indexing="ij")
        d = np.sqrt(P[0] ** 2 + P[1] ** 2 + P[2] ** 2)
        rhat = [np.where(d > 0, P[a] / np.where(d > 0, d, 1.0), 0.0) for a in range(3)]
        A2 = np.zeros_like(A0)
        for i, j in itertools.product(range(3), repeat=2):
            A2 += khat[i] * khat[j] * np.fft.fftn(rhat[i] * rhat[j] * F)
        A4 = np.zeros_like(A0)
        for i, j, k, l in itertools.product(range(3), repeat=4):
            A4 += khat[i] * khat[j] * khat[k] * khat[l] * np.fft.fftn(rhat[i] * rhat[j] * rhat[k] * rhat[l] * F)
        a0, a2, a4 = A0 / Wk, A2 / Wk, A4 / Wk
        c0 = np.abs(a0) ** 2 / norm - shot
        c2 = 2.5 * np.real(a0 * np.conj(3 * a2 - a0)) / norm
        c4 = 1.125 * np.real(a0 * np.conj(35 * a4 - 30 * a2 + 3 * a0)) / norm
    else:
        l = np.asarray(los, np.float64)
        l = l / np.linalg.norm(l)
        Pk = np.abs(A0 / Wk) ** 2 / norm
        mu = sum(khat[a] * l[a] for a in range(3))
        c0 = Pk - shot
        c2 = 5.0 * Pk * 0.5 * (3 * mu ** 2 - 1)
        c4 = 9.0 * Pk * 0.125 * (35 * mu ** 4 - 30 * mu ** 2 + 3)
    b = np.floor((kk - kmin) / dk).astype(np.int64)
    sel = (kk > 0) & (b >= 0) & (b < nbins)
    cnt = np.bincount(b[sel], minlength=nbins).astype(np.float64)

    def mean(v):
        s = np.bincount(b[sel], weights=v[sel], minlength=nbins)
        return np.where(cnt > 0, s / np.where(cnt > 0, cnt, 1.0), 0.0)

    return mean(kk), mean(c0), mean(c2), mean(c4), cnt.astype(np.int64), shot, norm
