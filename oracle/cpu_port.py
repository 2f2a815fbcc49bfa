"""The reference's CPU reconstruction path, restated in C (cpu_ref.c, OpenMP)
plus scipy.fft — the timed CPU baseline (test infrastructure, never the product).
A second solver, the GPU's FFT-preconditioned defect correction to a 1e-6
relative residual, can replace the reference's FMG schedule for a CPU timing
of the same work the GPU does.

One call of :meth:`CpuPort.lightcone_reconstruction` does what BAOrec.jl's
CPU path does for a lightcone with multigrid (``examples/lightcone_mg.jl``):
``reconstructed_potential!`` (paint data and randoms without wrapping, smooth
both, normalise, FMG with damped Jacobi — ``src/recon.jl:60-91, 184-212``,
``src/multigrid.jl:654-752``) and three ``reconstructed_positions`` calls
(data ``:sum``, randoms ``:sum`` and ``:disp``; ``src/recon.jl:264-388``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import scipy.fft as sfft

import baorec_oracle as O

F32 = np.float32
_P = C.c_void_p


class CpuPort:
    def __init__(self, threads=None):
        import build_oracle
        threads = threads or os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(threads))
        self.lib = C.CDLL(build_oracle.build())
        L = self.lib
        L.cpu_threads.restype = C.c_int
        L.cic_paint.argtypes = [_P, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, C.c_int64, _P, _P, C.c_int]
        L.read_cic.argtypes = [_P, C.c_int, C.c_int, C.c_int, _P, _P, _P, C.c_int64, _P, _P, _P]
        L.jacobi.argtypes = [_P, _P, _P, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, C.c_float, C.c_float, C.c_int]
        L.residual.argtypes = [_P, _P, _P, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, C.c_float]
        L.reduce.argtypes = [_P, _P, C.c_int, C.c_int, C.c_int]
        L.prolong.argtypes = [_P, _P, C.c_int, C.c_int, C.c_int, C.c_int]
        self.threads = int(L.cpu_threads())
        self.workers = threads

    # meshes are kept as flat x-fastest FP32 arrays ------------------------------
    @staticmethod
    def _p(a):
        return a.ctypes.data

    def paint(self, rho, n, x, y, z, w, bs, bm, wrap):
        x, y, z = (np.array(a, dtype=F32) for a in (x, y, z))
        w = np.ascontiguousarray(w, dtype=F32)
        L3 = np.asarray(bs, F32)
        B3 = np.asarray(bm, F32)
        st = self.lib.cic_paint(self._p(rho), n[0], n[1], n[2], self._p(x), self._p(y), self._p(z), self._p(w),
                                len(x), self._p(L3), self._p(B3), int(wrap))
        if st != 0:
            raise IndexError("paint index out of bounds (reference: BoundsError)")
        return rho

    def read(self, mesh, n, x, y, z, bs, bm):
        x, y, z = (np.ascontiguousarray(a, dtype=F32) for a in (x, y, z))
        out = np.empty(len(x), F32)
        L3 = np.asarray(bs, F32)
        B3 = np.asarray(bm, F32)
        self.lib.read_cic(self._p(mesh), n[0], n[1], n[2], self._p(x), self._p(y), self._p(z), len(x),
                          self._p(L3), self._p(B3), self._p(out))
        return out

    def _mesh3(self, flat, n):
        return flat.reshape((n[2], n[1], n[0])).transpose(2, 1, 0)

    def smooth(self, flat, n, R, bs):
        a = self._mesh3(flat, n)
        k = O.k_vec(n, bs, F32)
        fk = sfft.rfftn(a, axes=(2, 1, 0), workers=self.workers)
        k2 = O._k2(k, F32)
        fk *= np.exp(-0.5 * float(F32(R) * F32(R)) * k2.astype(np.float64)).astype(F32)
        out = sfft.irfftn(fk, s=(n[2], n[1], n[0]), axes=(2, 1, 0), workers=self.workers).astype(F32)
        return np.ascontiguousarray(out.transpose(2, 1, 0)).reshape(-1)

    def gradient(self, flat, n, bs):
        a = self._mesh3(flat, n)
        k = O.k_vec(n, bs, F32)
        pk = sfft.rfftn(a, axes=(2, 1, 0), workers=self.workers)
        kk = O._kk(k, None)
        out = []
        for i in range(3):
            g = sfft.irfftn((1j * kk[i]) * pk, s=(n[2], n[1], n[0]), axes=(2, 1, 0), workers=self.workers)
            out.append(np.ascontiguousarray(g.astype(F32).transpose(2, 1, 0)).reshape(-1))
        return out

    # multigrid ----------------------------------------------------------------
    def _tables(self, n, bs, bm):
        xv = O.x_vec(n, bs, bm, F32)
        return [np.ascontiguousarray(xv[a] / F32(F32(bs[a]) / F32(n[a])), dtype=F32) for a in range(3)]

    def fmg(self, f, n, bs, bm, beta, omega=0.4, nu=5, ncycles=6, los=None):
        L3 = np.asarray(bs, F32)
        los3 = None if los is None else np.asarray(los, F32)

        def rec(n):
            return all(v > 4 and v % 2 == 0 for v in n)

        def vcycle(v, f, n):
            P = self._tables(n, bs, bm)
            tmp = np.empty_like(v)
            args = (n[0], n[1], n[2], self._p(L3), self._p(P[0]), self._p(P[1]), self._p(P[2]),
                    None if los3 is None else self._p(los3))
            self.lib.jacobi(self._p(v), self._p(f), self._p(tmp), *args, F32(beta), F32(omega), nu)
            if rec(n):
                r = np.empty_like(v)
                self.lib.residual(self._p(r), self._p(v), self._p(f), *args, F32(beta))
                nc = tuple(s // 2 for s in n)
                f2 = np.empty(int(np.prod(nc)), F32)
                self.lib.reduce(self._p(f2), self._p(r), n[0], n[1], n[2])
                v2 = np.zeros_like(f2)
                vcycle(v2, f2, nc)
                self.lib.prolong(self._p(v), self._p(v2), n[0], n[1], n[2], 1)
            self.lib.jacobi(self._p(v), self._p(f), self._p(tmp), *args, F32(beta), F32(omega), nu)

        def fmg(f, n):
            if rec(n):
                nc = tuple(s // 2 for s in n)
                f2 = np.empty(int(np.prod(nc)), F32)
                self.lib.reduce(self._p(f2), self._p(f), n[0], n[1], n[2])
                v2 = fmg(f2, nc)
                v = np.empty_like(f)
                self.lib.prolong(self._p(v), self._p(v2), n[0], n[1], n[2], 0)
            else:
                v = np.zeros_like(f)
            for _ in range(ncycles):
                vcycle(v, f, n)
            return v

        return fmg(f, tuple(n))

    def solve_convergent(self, f, n, bs, bm, beta, rtol=1e-6):
        """The GPU's solver on the host: defect correction with the FFT
        preconditioner of the box's mean line of sight (oracle/fp64_oracle.py,
        FP64, C operator with OpenMP, scipy.fft with every core) until the
        relative residual is below rtol."""
        import fp64_oracle as P
        phi, _, hist = P.solve(self._mesh3(f, n), bs, bm, beta, None, rtol=rtol)
        self.last_history = hist
        return np.asarray(phi, dtype=np.float64).ravel(order="F").astype(F32)

    def lightcone_reconstruction(self, m, n, bs, bm, bias=2.0, growth=0.8, R=15.0, ran_min=0.01, solver="fmg"):
        """One reconstruction; returns (data :sum, randoms :sum, randoms :disp)
        positions.  solver "fmg" is the reference's schedule
        (src/multigrid.jl:722-752); "convergent" solves to a 1e-6 relative
        residual like the GPU's residual-driven solve."""
        N = int(np.prod(n))
        d = np.zeros(N, F32)
        r = np.zeros(N, F32)
        self.paint(d, n, m.x, m.y, m.z, m.w, bs, bm, False)
        self.paint(r, n, m.rx, m.ry, m.rz, m.rw, bs, bm, False)
        d = self.smooth(d, n, R, bs)
        r = self.smooth(r, n, R, bs)
        sd, sr = float(d.sum(dtype=np.float64)), float(r.sum(dtype=np.float64))
        al = F32(sd / sr)
        thr = F32(F32(ran_min) * F32(sr) / F32(len(m.rx)))
        d = d - al * r
        d = np.where(r > thr, d / np.where(r > thr, F32(bias) * al * r, F32(1)), F32(0)).astype(F32)
        beta = F32(F32(growth) / F32(bias))
        phi = self.fmg(d, n, bs, bm, beta) if solver == "fmg" else self.solve_convergent(d, n, bs, bm, beta)
        grads = self.gradient(phi, n, bs)
        out = []
        for (x, y, z), field in (((m.x, m.y, m.z), "sum"), ((m.rx, m.ry, m.rz), "sum"), ((m.rx, m.ry, m.rz), "disp")):
            disp = tuple(self.read(g, n, x, y, z, bs, bm) for g in grads)
            sh = O.read_shifts(disp, x, y, z, growth, los=None, field=field)
            out.append(O.reconstructed_positions(sh, x, y, z))
        return out
