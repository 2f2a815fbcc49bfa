"""Generate the known-answer fixtures in tests/golden/kat.npz.

The expected values are computed here from closed forms and exact rational
arithmetic, independently of the oracle, so that the oracle's restatement of
the reference can be checked against them:

* cic:   particles at dyadic positions on a mesh with a power-of-two cell
         (every FP32 operation of the reference formula is exact), expected
         CIC weights as exact fractions (src/mas.jl:13-49);
* smooth: a plane wave times exp(-R² k² / 2) (src/utils.jl:45-56);
* restrict: a periodic cosine times the full-weighting symbol
         ((1 + cos k h)/2 per axis) at the coarse centres 2c+1
         (src/multigrid.jl:520-584);
* prolong: a periodic cosine through trilinear interpolation
         (src/multigrid.jl:398-453);
* read:  a trilinear function read at dyadic positions (src/mas.jl:218-269);
* kvec:  2π i / L (src/utils.jl:3-10).

Run from the repository root: python tests/golden/make_golden.py
"""
import os
from fractions import Fraction as Fr

import numpy as np

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat.npz")


def cic_case():
    n, L = 8, 64.0               # cell 8: grid coordinates are dyadic
    pos = np.array([[23.5, 7.25, 40.0], [63.0, 0.5, 31.875], [0.0, 56.125, 12.5], [40.0, 40.0, 40.0]])
    w = np.array([1.0, 2.0, 0.5, 1.5])
    rho = {}
    for p, wt in zip(pos, w):
        idx, frac = [], []
        for a in range(3):
            g = Fr(p[a]).limit_denominator(1 << 20) * n / Fr(L) + 1
            c = int(g)           # floor for positive g
            w1 = g - c
            if c == n + 1:
                c = 1
            u = 1 if c == n else c + 1   # wrap = true
            idx.append((c - 1, u - 1))
            frac.append((1 - w1, w1))
        for dz in range(2):
            for dy in range(2):
                for dx in range(2):
                    key = (idx[0][dx], idx[1][dy], idx[2][dz])
                    val = Fr(wt).limit_denominator(16) * frac[0][dx] * frac[1][dy] * frac[2][dz]
                    rho[key] = rho.get(key, Fr(0)) + val
    mesh = np.zeros((n, n, n))
    for (i, j, k), v in rho.items():
        mesh[i, j, k] = float(v)
    return pos.astype(np.float32), w.astype(np.float32), mesh, np.array([L, L, L]), n


def main():
    out = {}
    pos, w, mesh, box, n = cic_case()
    out.update(cic_pos=pos, cic_w=w, cic_mesh=mesh, cic_box=box, cic_n=n)

    # smoothing of a plane wave
    n, L, R, m = 16, 200.0, 12.0, (3, 2, 1)
    x = np.arange(n) * L / n
    k = [2 * np.pi * mi / L for mi in m]
    wave = (np.cos(k[0] * x)[:, None, None] * np.cos(k[1] * x)[None, :, None] * np.cos(k[2] * x)[None, None, :])
    ksq = sum(v * v for v in k)
    out.update(sm_in=wave, sm_out=wave * np.exp(-0.5 * R * R * ksq), sm_L=L, sm_R=R)

    # restriction / prolongation of a cosine
    n, L, m = 16, 160.0, (1, 2, 3)
    h = L / n
    xf = np.arange(n) * h
    kk = [2 * np.pi * mi / L for mi in m]
    fine = (np.cos(kk[0] * xf)[:, None, None] * np.cos(kk[1] * xf)[None, :, None] * np.cos(kk[2] * xf)[None, None, :])
    xc = (2 * np.arange(n // 2) + 1) * h
    sym = np.prod([(1 + np.cos(v * h)) / 2 for v in kk])
    coarse = sym * (np.cos(kk[0] * xc)[:, None, None] * np.cos(kk[1] * xc)[None, :, None] * np.cos(kk[2] * xc)[None, None, :])
    out.update(rs_fine=fine, rs_coarse=coarse)
    # prolongation: exact trilinear interpolation of the coarse cosine samples
    cvals = (np.cos(kk[0] * xc)[:, None, None] * np.cos(kk[1] * xc)[None, :, None] * np.cos(kk[2] * xc)[None, None, :])
    nc = n // 2
    pro = np.zeros((n, n, n))
    def lerp_axis(vals_c, a):
        # fine index 2c+1 <- c; fine 2c+2 <- average of c and c+1 (periodic)
        res = np.zeros(vals_c.shape[:a] + (n,) + vals_c.shape[a + 1:])
        sl = [slice(None)] * 3
        for c in range(nc):
            sl[a] = c
            src = vals_c[tuple(sl)]
            sl[a] = (c + 1) % nc
            nxt = vals_c[tuple(sl)]
            sl[a] = 2 * c + 1
            res[tuple(sl)] = src
            sl[a] = (2 * c + 2) % n
            res[tuple(sl)] = 0.5 * (src + nxt)
        return res
    pro = lerp_axis(lerp_axis(lerp_axis(cvals, 0), 1), 2)
    out.update(pr_coarse=cvals, pr_fine=pro)

    # read-out of a trilinear function at dyadic positions (non-wrapping cells)
    n, L = 16, 128.0
    c = L / n
    ix = np.arange(n) * c
    a0, ax, ay, az = 0.5, 0.25, -0.125, 0.0625
    field = a0 + ax * ix[:, None, None] + ay * ix[None, :, None] + az * ix[None, None, :]
    rng = np.random.default_rng(5)
    p = (rng.integers(0, (n - 1) * 64, size=(200, 3)) / 64.0 * c).astype(np.float32)
    vals = a0 + ax * p[:, 0].astype(np.float64) + ay * p[:, 1] + az * p[:, 2]
    out.update(rd_field=field, rd_pos=p, rd_vals=vals, rd_L=L)

    # k axes
    n, L = 12, 300.0
    kx = 2 * np.pi * np.arange(n // 2 + 1) / L
    ky = 2 * np.pi * np.where(np.arange(n) < (n + 1) // 2, np.arange(n), np.arange(n) - n) / L
    out.update(kv_n=n, kv_L=L, kv_x=kx, kv_y=ky)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
