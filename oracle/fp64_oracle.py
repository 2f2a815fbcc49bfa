"""FP64 accuracy judge at full mesh sizes (test infrastructure, never the product).

The relative L2 error of the displacement field is quoted against an FP64
solution of the same discrete system the FP32 code solves: the multigrid
operator of ``src/multigrid.jl:14-135, 213-326`` with its coefficients
rounded to FP32 exactly as :func:`baorec_oracle.stencil_coefficients` rounds
them, applied in FP64 arithmetic.  :func:`baorec_oracle.solve_mg` computes
that solution with V-cycles in NumPy, which takes minutes at 256^3; this
module evaluates the same operator in C (``apply_op_f64`` in ``cpu_ref.c``,
OpenMP) and iterates with an FFT preconditioner in FP64, so a 256^3 solve to
a 1e-11 relative residual takes seconds to a minute on a host's cores.

The solver is a defect correction with a scalar shift, as the periodic
operator is singular (``A·1 = 0``) and its left null vector is not constant
for the radial line of sight::

    r = f - α - A φ;  α += mean(r);  φ += S⁻¹ (r - mean(r))

with ``S(k)`` the Fourier symbol of the operator for one fixed line of sight
``l`` (the direction of the box centre for the radial line of sight):
``Σ_a (1 + β l_a²)/c_a² · 4 sin²(θ_a/2) + Σ_{a<b} 2β l_a l_b/(c_a c_b) sin θ_a sin θ_b``.
The answer does not depend on the preconditioner: the loop stops on the FP64
residual of the exact operator.  ``tests/test_fp64_oracle.py`` pins the C
operator to :func:`baorec_oracle.apply_operator` and the solution to
:func:`baorec_oracle.solve_mg` at small sizes.

Meshes are NumPy arrays indexed ``[ix, iy, iz]``; they are kept in Fortran
order (x fastest) so that the C code sees the layout ``ix + n1 (iy + n2 iz)``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import scipy.fft as sfft

import baorec_oracle as O
import build_oracle

F32 = np.float32
_P = C.c_void_p
_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        lib = C.CDLL(build_oracle.build())
        lib.apply_op_f64.argtypes = [_P, _P, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, C.c_float]
        lib.apply_op_f64.restype = None
        _LIB = lib
    return _LIB


def _workers():
    return os.cpu_count() or 1


class Operator:
    """The multigrid operator of one mesh and box (FP32 coefficients, FP64
    arithmetic).  ``los=None`` is the radial line of sight from the origin."""

    def __init__(self, shape, box_size, box_min, beta, los=None):
        self.shape = tuple(int(s) for s in shape)
        self.beta = F32(beta)
        self.L = np.asarray(box_size, F32).copy()
        self.bmin = np.asarray(box_min, F32).copy()
        self.los = None if los is None else np.asarray(los, F32).copy()
        n = self.shape
        xv = O.x_vec(n, self.L, self.bmin, F32)
        # p = x_vec / cell per axis (src/multigrid.jl:17-21), FP32 as the oracle rounds it
        self.P = [np.ascontiguousarray(xv[a] / F32(F32(self.L[a]) / F32(n[a])), dtype=F32) for a in range(3)]

    def apply(self, v):
        v = np.asfortranarray(v, dtype=np.float64)
        out = np.empty(self.shape, dtype=np.float64, order="F")
        los = None if self.los is None else self.los.ctypes.data
        _lib().apply_op_f64(out.ctypes.data, v.ctypes.data, *self.shape, self.L.ctypes.data,
                            self.P[0].ctypes.data, self.P[1].ctypes.data, self.P[2].ctypes.data, los,
                            self.beta)
        return out

    def symbol_inverse(self):
        """1/S(k) on the rfftn grid of :func:`baorec_oracle.rfft3` (axis 0 halved)."""
        n = self.shape
        cell = [float(self.L[a]) / n[a] for a in range(3)]
        if self.los is None:
            centre = self.bmin.astype(np.float64) + 0.5 * self.L.astype(np.float64)
            nrm = np.linalg.norm(centre)
            l = centre / nrm if nrm > 0 else np.zeros(3)
        else:
            l = self.los.astype(np.float64)
            l = l / max(np.linalg.norm(l), 1e-300)
        b = float(self.beta)
        th = [2 * np.pi * np.fft.rfftfreq(n[0]) , 2 * np.pi * np.fft.fftfreq(n[1]), 2 * np.pi * np.fft.fftfreq(n[2])]
        shp = [(-1, 1, 1), (1, -1, 1), (1, 1, -1)]
        s2 = [(4 * np.sin(th[a] / 2) ** 2).reshape(shp[a]) for a in range(3)]
        s1 = [np.sin(th[a]).reshape(shp[a]) for a in range(3)]
        S = sum((1 + b * l[a] ** 2) / cell[a] ** 2 * s2[a] for a in range(3))
        for a in range(3):
            for c in range(a + 1, 3):
                S = S + 2 * b * l[a] * l[c] / (cell[a] * cell[c]) * s1[a] * s1[c]
        S = np.broadcast_to(S, (n[0] // 2 + 1, n[1], n[2]))
        with np.errstate(divide="ignore"):
            inv = np.where(S > 0, 1.0 / np.where(S > 0, S, 1.0), 0.0)
        inv[0, 0, 0] = 0.0
        return inv

    def precondition(self, r, inv):
        rk = sfft.rfftn(r, axes=(2, 1, 0), workers=_workers())
        rk *= inv
        return np.asfortranarray(sfft.irfftn(rk, s=(self.shape[2], self.shape[1], self.shape[0]),
                                             axes=(2, 1, 0), workers=_workers()))


def solve(f, box_size, box_min, beta, los=None, rtol=1e-11, max_iter=200, phi0=None):
    """FP64 solution of ``A φ = f - α`` (the residual-driven multigrid's
    system); returns ``(φ, α, history)`` with history the relative residual
    ``|f - α - A φ| / |f - α|`` before each correction."""
    f = np.asfortranarray(f, dtype=np.float64)
    op = Operator(f.shape, box_size, box_min, beta, los)
    inv = op.symbol_inverse()
    phi = np.zeros_like(f) if phi0 is None else np.asfortranarray(phi0, dtype=np.float64).copy()
    alpha = float(np.mean(f))
    hist = []
    for _ in range(max_iter + 1):
        r = f - alpha - op.apply(phi)
        fn = float(np.linalg.norm(f - alpha))
        hist.append(float(np.linalg.norm(r)) / fn)
        if hist[-1] <= rtol:
            break
        m = float(np.mean(r))
        alpha += m
        r -= m
        phi += op.precondition(r, inv)
    else:
        raise RuntimeError(f"FP64 oracle solve did not reach {rtol}: {hist[-5:]}")
    return phi, alpha, hist


def gradient_meshes(phi, box_size):
    """``∂_i φ = irfft(i k_i φ_k)`` in FP64 (``src/multigrid.jl:755-773``)."""
    n = phi.shape
    k = O.k_vec(n, box_size, np.float64)
    pk = sfft.rfftn(phi, axes=(2, 1, 0), workers=_workers())
    kk = O._kk(k, None)
    return tuple(sfft.irfftn((1j * kk[i]) * pk, s=(n[2], n[1], n[0]), axes=(2, 1, 0), workers=_workers())
                 for i in range(3))


def rel_l2_vector(a, b):
    """Relative L2 error of a vector field (three meshes) against ``b``."""
    num = sum(float(np.linalg.norm(np.asarray(a[i], np.float64) - np.asarray(b[i], np.float64)) ** 2)
              for i in range(3))
    den = sum(float(np.linalg.norm(np.asarray(b[i], np.float64)) ** 2) for i in range(3))
    return float(np.sqrt(num / den))
