"""Cosmology on the host and catalog coordinates on the device.

``Cosmology`` restates ``src/cosmo.jl:19-81`` (BAOrec.jl): the density
parameters are evaluated in FP32 from the same inputs as the Julia struct
(whose field type follows ``ω_b::Float32``), E(z) and the comoving distance
in FP64.  The reference tabulates r(z) = c ∫ dz / H(z) with one adaptive
quadrature per table point (``quadgk``, rtol 1e-8); here the table comes from
a cumulative composite Simpson rule on a grid 8x finer than the table, which
agrees with the quadrature to far below FP32 resolution.

``sky_to_cartesian``, ``cartesian_to_sky`` and ``fkp_weights`` are the
lightcone scripts' conversions (``examples/lightcone.jl:30-82``) run on the
GPU through ``baorec_sky_to_cartesian`` / ``baorec_cartesian_to_sky`` /
``baorec_fkp_weights``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib

F32 = np.float32
SPEED_OF_LIGHT = 299792.458          # km/s
_G = 6.67408e-11
_MPC = 3.085677581491367e22
_HBAR = 6.582119514e-16
_EVC2 = 1.782661907e-36
_KB = 8.6173303e-5


@dataclass
class Cosmology:
    """``Cosmology`` of src/cosmo.jl:19-70 (FP32 parameters as in Julia)."""
    omega_b: float = 0.0225
    omega_c: float = 0.12
    h: float = 0.67
    Neff: float = 3.044
    Omega_k0: float = 0.0
    T_cmb: float = 2.725
    w0: float = -1.0
    wa: float = 0.0
    ns: float = 0.96
    z_tab_min: float = 0.0
    z_tab_max: float = 3.0
    z_tab_num: int = 100000
    _table: object = field(default=None, repr=False)

    def __post_init__(self):
        h = F32(self.h)
        h2 = F32(h * h)
        self.H0 = F32(h * F32(100))
        rho_g0 = F32(3 * 100 ** 2 / (8 * np.pi * _G) * _HBAR ** 3 * (1.0 / (1e-3 * _MPC)) ** 2 * (1.0 / _EVC2)
                     * (SPEED_OF_LIGHT * 1e3) ** 3)
        self.Omega_g0 = F32((np.pi ** 2 / 15) * (2.725 * _KB) ** 4 / float(rho_g0) * (float(F32(self.T_cmb)) / 2.725) ** 4
                            / float(h2))
        self.Omega_nu0 = F32(float(F32(self.Neff)) * (7 / 8 * (4 / 11) ** (4 / 3)) * float(self.Omega_g0))
        self.Omega_b0 = F32(F32(self.omega_b) / h2)
        self.Omega_c0 = F32(F32(self.omega_c) / h2)
        self.Omega_L0 = F32(F32(1) - F32(self.Omega_k0) - self.Omega_b0 - self.Omega_c0 - self.Omega_nu0 - self.Omega_g0)
        self.Omega_m0 = F32(self.Omega_b0 + self.Omega_c0)

    def E(self, z):
        """E(z) of src/cosmo.jl:77 in FP64."""
        z = np.asarray(z, np.float64)
        a = 1.0 / (1.0 + z)
        with np.errstate(divide="ignore", invalid="ignore"):
            fde = -3 * (1 + float(self.w0)) + 3 * float(self.wa) * ((a - 1) / np.log(a) - 1)
        fde = np.where(z == 0, 0.0, fde) if float(self.wa) != 0.0 else -3 * (1 + float(self.w0)) + 0 * z
        ol = float(self.Omega_L0) * (1 + z) ** (-fde)
        return np.sqrt((float(self.Omega_nu0) + float(self.Omega_g0)) * (1 + z) ** 4
                       + (float(self.Omega_b0) + float(self.Omega_c0)) * (1 + z) ** 3
                       + float(self.Omega_k0) * (1 + z) ** 2 + ol)

    def H(self, z):
        return float(F32(self.h)) * 100 * self.E(z)

    def distance_table(self):
        """(z grid, comoving distance in Mpc) as comoving_distance_interp tabulates it."""
        if self._table is None:
            n = int(self.z_tab_num)
            zg = np.linspace(float(self.z_tab_min), float(self.z_tab_max), n)
            fine = 8
            zf = np.linspace(float(self.z_tab_min), float(self.z_tab_max), (n - 1) * fine + 1)
            inv = SPEED_OF_LIGHT / self.H(zf)
            # cumulative Simpson over pairs of fine intervals
            hstep = zf[1] - zf[0]
            pair = hstep / 3 * (inv[:-2:2] + 4 * inv[1:-1:2] + inv[2::2])
            cum = np.concatenate([[0.0], np.cumsum(pair)])          # at even fine nodes
            r = cum[:: fine // 2]
            if float(self.z_tab_min) != 0.0:
                r = r + self.comoving_distance(float(self.z_tab_min))
            self._table = (zg, r)
        return self._table

    def comoving_distance(self, z):
        from scipy.integrate import quad
        return SPEED_OF_LIGHT * quad(lambda u: 1.0 / self.H(u), 0.0, z, epsrel=1e-10)[0]


def DESICosmology(**kw) -> Cosmology:
    """src/cosmo.jl:72-74."""
    args = dict(omega_b=0.02237, omega_c=0.1200, h=0.6736, ns=0.9649, Neff=2.0328 + 1.0, w0=-1.0, wa=0.0)
    args.update(kw)
    return Cosmology(**args)


def _ctx():
    from .recon import _prim_ctx
    return _prim_ctx((2, 2, 2), [1.0] * 3, [0.0] * 3)


def _call3(name, a, b, c, cosmo, h):
    import torch
    zg, r = cosmo.distance_table()
    table = np.ascontiguousarray(r, np.float64)
    dev = isinstance(a, torch.Tensor) and a.is_cuda
    n = int(a.numel() if dev else len(a))
    ctx = _ctx()
    if dev:
        ins = [t.contiguous() for t in (a, b, c)]
        outs = [torch.empty(n, device=a.device, dtype=torch.float32) for _ in range(3)]
        ptr = lambda t: t.data_ptr()
        flags = 0
    else:
        ins = [np.ascontiguousarray(v, F32) for v in (a, b, c)]
        outs = [np.empty(n, F32) for _ in range(3)]
        ptr = lambda t: t.ctypes.data
        flags = _lib.HOST
    ctx.call(name, *[ptr(t) for t in ins], n, table.ctypes.data, len(table), float(zg[0]), float(zg[-1]), float(h),
             *[ptr(t) for t in outs], flags)
    return tuple(outs)


def sky_to_cartesian(ra, dec, z, cosmo: Cosmology):
    """examples/lightcone.jl:30-47 → (x, y, z) in Mpc/h (FP32 arrays)."""
    # the script scales by h = H₀ / 100 in FP32
    return _call3("baorec_sky_to_cartesian", ra, dec, z, cosmo, float(F32(cosmo.H0 / F32(100))))


def cartesian_to_sky(x, y, z, cosmo: Cosmology):
    """examples/lightcone.jl:50-80 → (ra, dec, redshift); ra in (-360, 0] as the script returns it."""
    # the script divides by cosmo.h
    return _call3("baorec_cartesian_to_sky", x, y, z, cosmo, float(F32(cosmo.h)))


def fkp_weights(nz, P0):
    """examples/lightcone.jl:82: 1 / (1 + nz P0)."""
    nz = np.ascontiguousarray(nz, F32)
    w = np.empty_like(nz)
    _ctx().call("baorec_fkp_weights", nz.ctypes.data, len(nz), float(P0), w.ctypes.data, _lib.HOST)
    return w
