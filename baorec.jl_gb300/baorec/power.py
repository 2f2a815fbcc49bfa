"""Power-spectrum multipoles on the GPU (``baorec_power_multipoles``): the
science check the reference's test helpers run with the external pypowspec
(``compute_auto_box``, ``compute_auto_box_rand``, ``compute_auto_lc``;
``test_helpers/simulation.py:40-55``, ``test_helpers/lightcone.py:48-75``).
The same names are kept; the configuration that pypowspec reads from a
``.conf`` file is passed as keyword arguments.  Each call returns a dict
with ``k`` (mean |k| of the shell's modes), ``multipoles`` (nbins x 3:
P_0, P_2, P_4), ``nmodes``, ``shot_noise`` and ``norm``."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

F32 = np.float32


def _is_dev(a):
    try:
        import torch
        return isinstance(a, torch.Tensor) and a.is_cuda
    except ImportError:
        return False


def _arrays(arrs):
    dev = {(_is_dev(a)) for a in arrs if a is not None}
    if len(dev) > 1:
        raise TypeError("catalog arrays must be all host (NumPy) or all device (CUDA torch)")
    dev = bool(dev and dev.pop())
    keep, ptrs = [], []
    for a in arrs:
        if a is None:
            ptrs.append(None)
        elif dev:
            t = a.contiguous().float()
            keep.append(t)
            ptrs.append(t.data_ptr())
        else:
            h = np.ascontiguousarray(a, dtype=F32)
            keep.append(h)
            ptrs.append(h.ctypes.data)
    return dev, keep, ptrs


def _bins(kmin, kmax, bin_size, box_size, grid_size):
    if kmax is None:
        kmax = min(np.pi * g / L for g, L in zip(grid_size, box_size))   # Nyquist
    nb = int(np.floor((kmax - kmin) / bin_size + 1e-9))
    if nb < 1:
        raise ValueError("no k bins between kmin and kmax")
    return nb


def multipoles(x, y, z, w=None, rx=None, ry=None, rz=None, rw=None, rnz=None, *, geometry="box", box_size=1000.0,
               box_min=0.0, grid_size=256, mas="tsc", interlace=None, los=(0.0, 0.0, 1.0), kmin=0.0, kmax=None,
               bin_size=0.005):
    """P_0, P_2, P_4 of the data (minus alpha times the randoms, if given) on
    a grid_size^3 mesh over [box_min, box_min + box_size)^3; geometry "box"
    (periodic, fixed line of sight) or "survey" (line of sight from the
    origin, needs randoms and their n(z))."""
    from .recon import _prim_ctx
    L = [float(v) for v in np.broadcast_to(np.asarray(box_size, np.float64), 3)]
    bm = [float(v) for v in np.broadcast_to(np.asarray(box_min, np.float64), 3)]
    g = tuple(int(v) for v in np.broadcast_to(np.asarray(grid_size), 3))
    geo = {"box": _lib.POWER_BOX, "survey": _lib.POWER_SURVEY}[geometry]
    if interlace is None:
        interlace = geometry == "box"
    nb = _bins(kmin, kmax, bin_size, L, g)
    pc = _lib.PowerConfig()
    pc.geometry, pc.mas, pc.interlace, pc.nbins = geo, {"cic": _lib.MAS_CIC, "tsc": _lib.MAS_TSC}[mas], int(interlace), nb
    pc.kmin, pc.dk = float(kmin), float(bin_size)
    for a in range(3):
        pc.los[a] = float(los[a])
    dev, keep, ptrs = _arrays([x, y, z, w, rx, ry, rz, rw, rnz])
    n = int(len(x))
    nr = 0 if rx is None else int(len(rx))
    ctx = _prim_ctx(g, L, bm)
    if dev:
        import torch
        torch.cuda.synchronize()
    out = [np.zeros(nb) for _ in range(4)]
    nm = np.zeros(nb, np.int64)
    shot, norm = C.c_double(), C.c_double()
    ctx.call("baorec_power_multipoles", C.byref(pc), *ptrs[:4], n, *ptrs[4:9], nr,
             *[o.ctypes.data for o in out], nm.ctypes.data, C.byref(shot), C.byref(norm),
             0 if dev else _lib.HOST)
    del keep
    return {"k": out[0], "multipoles": np.stack(out[1:], axis=1), "nmodes": nm, "shot_noise": shot.value,
            "norm": norm.value}


def compute_auto_box(x, y, z, w=None, **kw):
    """Periodic box, data only (pypowspec ``compute_auto_box``)."""
    return multipoles(x, y, z, w, geometry="box", **kw)


def compute_auto_box_rand(x, y, z, w, rx, ry, rz, rw=None, **kw):
    """Periodic box, data minus randoms (pypowspec ``compute_auto_box_rand``)."""
    return multipoles(x, y, z, w, rx, ry, rz, rw, geometry="box", **kw)


def compute_auto_lc(x, y, z, w, nz, rx, ry, rz, rw, rnz, box_pad=0.02, **kw):
    """Survey (pypowspec ``compute_auto_lc``) on Cartesian comoving positions
    (``baorec.cosmo.sky_to_cartesian`` converts RA, Dec, z); w are the total
    weights (completeness x FKP).  Without box_size/box_min the mesh box is
    the randoms' bounding cube enlarged by box_pad on each side."""
    if "box_size" not in kw or "box_min" not in kw:
        lo = np.array([float(np.min(np.asarray(a.cpu() if _is_dev(a) else a))) for a in (rx, ry, rz)])
        hi = np.array([float(np.max(np.asarray(a.cpu() if _is_dev(a) else a))) for a in (rx, ry, rz)])
        side = float(np.max(hi - lo)) * (1 + 2 * box_pad)
        kw.setdefault("box_size", side)
        kw.setdefault("box_min", list((lo + hi) / 2 - side / 2))
    del nz   # the data's n(z) is not needed: the normalisation uses the randoms'
    return multipoles(x, y, z, w, rx, ry, rz, rw, rnz, geometry="survey", **kw)
