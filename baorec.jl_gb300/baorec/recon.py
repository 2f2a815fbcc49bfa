"""Python mirror of BAOrec.jl's reconstruction API over the GB300 library.

Names follow the Julia package (``src/BAOrec.jl:22-25``, ``src/recon.jl``);
Julia's mutating ``f!`` becomes ``f_`` (trailing underscore).  Arrays are
either NumPy arrays (host; the reference's ``Array`` methods) or CUDA torch
tensors (device; the reference's ``CuArray`` methods).  Every computation runs
in the CUDA library; there is no CPU path.

Meshes are indexed ``[ix, iy, iz]`` (0-based) with x fastest in memory, i.e.
NumPy arrays of shape ``(n1, n2, n3)`` in Fortran order, or torch tensors
created by :func:`zeros_mesh`.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field as dc_field
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import BaorecError, BoundsError, NotConverged  # noqa: F401

__all__ = [
    "IterativeRecon", "MultigridRecon", "run_", "setup_fft_", "setup_overdensity_",
    "reconstructed_overdensity_", "reconstructed_potential_", "read_shifts",
    "reconstructed_positions", "reconstructed_positions2", "k_vec", "x_vec", "setup_box", "cic_", "tsc_", "cell_bins",
    "read_cic_", "smooth_", "iterate_", "jacobi_", "residual_", "reduce_", "prolong_",
    "vcycle_", "fmg", "solve_", "compute_displacements", "zeros_mesh", "BaorecError",
    "BoundsError", "NotConverged",
]

F32 = np.float32


def _torch():
    import torch
    return torch


def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


@dataclass
class IterativeRecon:
    """``IterativeRecon`` (``src/recon.jl:2-16``)."""
    bias: float
    f: float
    smoothing_radius: float
    box_size: Optional[Sequence[float]] = None
    box_min: Optional[Sequence[float]] = None
    los: Optional[Sequence[float]] = None
    n_iter: int = 3
    beta: Optional[float] = None
    fft_plan: object = None
    result_cache: object = None
    mas: str = "cic"                     # addition: "cic" | "tsc"
    deterministic: bool = False          # paint through the tile counting sort (bit-reproducible mesh)

    def __post_init__(self):
        if self.beta is None:            # β = typeof(bias)(f / bias)
            self.beta = float(F32(F32(self.f) / F32(self.bias)))


_STARTS = {"zero": _lib.START_ZERO, "spectral": _lib.START_SPECTRAL, "learned": _lib.START_LEARNED}


@dataclass
class MultigridRecon:
    """``MultigridRecon`` (``src/recon.jl:18-33``) plus the residual-driven
    solver options (``mg_mode="convergent"``)."""
    bias: float
    f: float
    smoothing_radius: float
    box_size: Optional[Sequence[float]] = None
    box_min: Optional[Sequence[float]] = None
    los: Optional[Sequence[float]] = None
    jacobi_damping_factor: float = 0.4
    jacobi_niterations: int = 5
    vcycle_niterations: int = 6
    beta: Optional[float] = None
    fft_plan: object = None
    result_cache: object = None
    mas: str = "cic"
    deterministic: bool = False          # paint through the tile counting sort (bit-reproducible mesh)
    mg_mode: str = "reference"           # "reference" (FMG schedule) | "convergent"
    nu1: int = 2
    nu2: int = 2
    rtol: float = 1e-6
    max_cycles: int = 50
    start: str = "zero"                  # convergent mode: "zero" | "spectral" | "learned"
    start_rate: float = 0.5
    guess_params: object = None          # learned start: network parameters (baorec.guess)
    guess_level: int = 0                 # learned start: 0 network on this mesh, 1 on its first restriction
    gradient: str = "fft"                # displacement from φ: "fft" (reference) | "fd" (central differences)
    solve_stats: dict = dc_field(default_factory=dict)

    def __post_init__(self):
        if self.beta is None:
            self.beta = float(F32(F32(self.f) / F32(self.bias)))
        if self.start not in _STARTS:
            raise ValueError(f"start must be one of {sorted(_STARTS)}, got {self.start!r}")
        if self.start == "learned" and self.guess_params is None:
            raise ValueError("start='learned' needs guess_params (see baorec.guess)")
        if self.gradient not in ("fft", "fd"):
            raise ValueError(f"gradient must be 'fft' or 'fd', got {self.gradient!r}")


# ----------------------------------------------------------------------------
# argument marshalling
# ----------------------------------------------------------------------------

class _Particles:
    """Contiguous FP32 views of particle arrays and the host/device flag."""

    def __init__(self, *arrays):
        self.keep = []
        self.orig = arrays
        kinds = {(_is_torch(a) and a.is_cuda) for a in arrays if a is not None}
        if len(kinds) > 1:
            raise TypeError("particle arrays must be all host (NumPy) or all device (CUDA torch)")
        self.device = bool(kinds and kinds.pop())
        self.ptrs = []
        self.n = None
        for a in arrays:
            if a is None:
                self.ptrs.append(None)
                continue
            if self.device:
                t = a
                if t.dtype != _torch().float32 or not t.is_contiguous():
                    t = t.to(_torch().float32).contiguous()
                self.keep.append(t)
                self.ptrs.append(t.data_ptr())
                n = t.numel()
            else:
                h = np.ascontiguousarray(a, dtype=F32)
                self.keep.append(h)
                self.ptrs.append(h.ctypes.data)
                n = h.size
            if self.n is None:
                self.n = n
        self.flags = 0 if self.device else _lib.HOST

    def writeback(self, i):
        """Copy a (possibly staged) array back into the caller's array i."""
        src, dst = self.keep[i], self.orig[i]
        if src is dst:
            return
        if self.device:
            dst.copy_(src)
        elif isinstance(dst, np.ndarray) and dst.flags.writeable:
            dst[...] = src


def _sync_torch():
    try:
        torch = _torch()
        if torch.cuda.is_available() and torch.cuda.is_initialized():
            torch.cuda.synchronize()
    except ImportError:
        pass


class _Mesh:
    """Device pointer for a mesh argument; NumPy meshes are staged through a
    CUDA tensor and copied back on exit when written."""

    def __init__(self, a, shape=None, write=True):
        self.a = a
        self.write = write
        torch = _torch()
        if _is_torch(a):
            if not a.is_cuda or a.dtype != torch.float32:
                raise TypeError("device meshes must be CUDA float32 tensors")
            self.shape = tuple(a.shape)
            if not a.permute(2, 1, 0).is_contiguous():
                raise ValueError("device mesh must be x-fastest (create it with zeros_mesh)")
            self.t = a
        else:
            h = np.asarray(a)
            self.shape = h.shape
            self.t = torch.from_numpy(np.ascontiguousarray(h.astype(F32).transpose(2, 1, 0))).cuda()
        self.ptr = self.t.data_ptr()

    def __enter__(self):
        _sync_torch()
        return self

    def __exit__(self, *exc):
        if exc[0] is None and self.write and not _is_torch(self.a):
            out = self.t.cpu().numpy().transpose(2, 1, 0)
            self.a[...] = out
        return False


def zeros_mesh(shape, device: bool = True):
    """A zero FP32 mesh of shape (n1, n2, n3), x fastest: a CUDA tensor
    (``device=True``) or a Fortran-ordered NumPy array."""
    n1, n2, n3 = shape
    if device:
        torch = _torch()
        return torch.zeros((n3, n2, n1), dtype=torch.float32, device="cuda").permute(2, 1, 0)
    return np.zeros(shape, dtype=F32, order="F")


def _empty_like_kind(shape, device):
    return zeros_mesh(shape, device=device)


def _vec_out(n, device):
    if device:
        return _torch().empty(n, dtype=_torch().float32, device="cuda")
    return np.empty(n, dtype=F32)


def _vptr(a):
    return a.data_ptr() if _is_torch(a) else a.ctypes.data


# ----------------------------------------------------------------------------
# contexts (the reference's fft_plan slot holds one)
# ----------------------------------------------------------------------------

def _config(recon, shape, ran_min=0.01) -> _lib.Config:
    c = _lib.default_config()
    c.ran_min = float(ran_min)
    mg = isinstance(recon, MultigridRecon)
    c.method = _lib.MULTIGRID if mg else _lib.ITERATIVE
    for a in range(3):
        c.n[a] = int(shape[a])
    bs = recon.box_size if recon.box_size is not None else [1.0, 1.0, 1.0]
    bm = recon.box_min if recon.box_min is not None else [0.0, 0.0, 0.0]
    for a in range(3):
        c.box_size[a] = float(bs[a])
        c.box_min[a] = float(bm[a])
    if recon.los is None:
        c.los_mode = _lib.LOS_LOCAL
    else:
        c.los_mode = _lib.LOS_GLOBAL
        for a in range(3):
            c.los[a] = float(recon.los[a])
    c.bias = float(recon.bias)
    c.f = float(recon.f)
    c.smoothing_radius = float(recon.smoothing_radius)
    c.beta = float(recon.beta)
    c.mas = _lib.MAS_TSC if recon.mas == "tsc" else _lib.MAS_CIC
    if mg:
        c.jacobi_damping_factor = float(recon.jacobi_damping_factor)
        c.jacobi_niterations = int(recon.jacobi_niterations)
        c.vcycle_niterations = int(recon.vcycle_niterations)
        c.mg_mode = _lib.MG_CONVERGENT if recon.mg_mode == "convergent" else _lib.MG_REFERENCE
        c.nu1, c.nu2 = int(recon.nu1), int(recon.nu2)
        c.rtol = float(recon.rtol)
        c.max_cycles = int(recon.max_cycles)
        c.mg_start = _STARTS[recon.start]
        c.start_rate = float(recon.start_rate)
    else:
        c.n_iter = int(recon.n_iter)
    return c


def _same(a: _lib.Config, b: _lib.Config, ignore_box=True) -> bool:
    for name, _ in _lib.Config._fields_:
        if ignore_box and name in ("box_size", "box_min"):
            continue
        va, vb = getattr(a, name), getattr(b, name)
        if hasattr(va, "__len__"):
            if list(va) != list(vb):
                return False
        elif va != vb:
            return False
    return True


def setup_fft_(recon, field_or_shape):
    """``setup_fft!`` (``src/recon.jl:35-37``): create (or reuse) the context
    holding the cuFFT plans and buffers for this mesh size."""
    shape = tuple(field_or_shape.shape) if hasattr(field_or_shape, "shape") else tuple(field_or_shape)
    return _ctx(recon, shape)


def _ctx(recon, shape, ran_min=0.01) -> _lib.Context:
    cfg = _config(recon, shape, ran_min)
    ctx = recon.fft_plan
    if not isinstance(ctx, _lib.Context) or not _same(ctx.cfg, cfg):
        if isinstance(ctx, _lib.Context):
            ctx.close()
        ctx = _lib.Context(cfg)
        recon.fft_plan = ctx
        if getattr(recon, "guess_params", None) is not None:
            ctx.call("baorec_guess_set_level", int(getattr(recon, "guess_level", 0)))
            p = np.ascontiguousarray(recon.guess_params, dtype=np.float32)
            ctx.call("baorec_guess_set_params", p.ctypes.data, p.size)
    elif recon.box_size is not None and recon.box_min is not None:
        bs, bm = ctx.box()
        if list(bs) != [float(F32(v)) for v in recon.box_size] or list(bm) != [float(F32(v)) for v in recon.box_min]:
            ctx.set_box(recon.box_size, recon.box_min)
    if isinstance(recon, MultigridRecon):
        ctx.call("baorec_set_gradient", 1 if recon.gradient == "fd" else 0)
    return ctx


_PRIM_CACHE = {}


def _prim_ctx(shape, box_size, box_min, **kw) -> _lib.Context:
    """Context for the stand-alone mesh primitives (cic!, smooth!, ...)."""
    kw.setdefault("bias", 1.0)
    kw.setdefault("f", 0.0)
    kw.setdefault("smoothing_radius", 0.0)
    mg = kw.pop("multigrid", False)
    cls = MultigridRecon if mg else IterativeRecon
    rec = cls(box_size=box_size, box_min=box_min, **kw)
    key = (tuple(shape), mg, tuple(sorted((k, str(v)) for k, v in kw.items())))
    holder = _PRIM_CACHE.get(key)
    if holder is None:
        holder = rec
        _PRIM_CACHE[key] = holder
    holder.box_size, holder.box_min = box_size, box_min
    return _ctx(holder, shape)


def _result_to(ctx, like_device, shape):
    out = _empty_like_kind(shape, like_device)
    if like_device:
        _sync_torch()
        ctx.call("baorec_get_result", C.c_void_p(out.data_ptr()), 0)
    else:
        tmp = np.empty(int(np.prod(shape)), dtype=F32)
        ctx.call("baorec_get_result", C.c_void_p(tmp.ctypes.data), _lib.HOST)
        out[...] = tmp.reshape(shape, order="F")
    return out


# ----------------------------------------------------------------------------
# grid utilities — src/utils.jl
# ----------------------------------------------------------------------------

def k_vec(field_or_dims, box_size):
    """``k_vec`` (``src/utils.jl:3-10``): (rfftfreq, fftfreq, fftfreq) axes."""
    dims = field_or_dims.shape if hasattr(field_or_dims, "shape") else field_or_dims
    out = []
    for a, n in enumerate(dims):
        fs = F32(2.0 * np.pi * n / float(box_size[a]))
        mult = F32(fs / F32(n))
        idx = np.arange(n // 2 + 1) if a == 0 else np.where(np.arange(n) < (n + 1) // 2, np.arange(n), np.arange(n) - n)
        out.append(idx.astype(F32) * mult)
    return tuple(out)


def x_vec(field_or_dims, box_size, box_min):
    """``x_vec`` (``src/utils.jl:21-25``): cell-centre axes."""
    dims = field_or_dims.shape if hasattr(field_or_dims, "shape") else field_or_dims
    out = []
    for a, n in enumerate(dims):
        cell = float(F32(F32(box_size[a]) / F32(n)))
        out.append((float(box_min[a]) + (np.arange(n) + 0.5) * cell).astype(F32))
    return tuple(out)


def setup_box(x, y, z, box_pad):
    """``setup_box`` (``src/utils.jl:100-109``) as a device min/max reduction."""
    p = _Particles(x, y, z)
    ctx = _prim_ctx((2, 2, 2), [1, 1, 1], [0, 0, 0])
    bs, bm = _lib.F3(), _lib.F3()
    ctx.call("baorec_setup_box", p.ptrs[0], p.ptrs[1], p.ptrs[2], p.n, float(box_pad), p.flags, bs, bm)
    return np.array(list(bs), dtype=F32), np.array(list(bm), dtype=F32)


# ----------------------------------------------------------------------------
# mass assignment — src/mas.jl
# ----------------------------------------------------------------------------

def _paint(name, rho, x, y, z, w, box_size, box_min, wrap, deterministic=False, binned=None):
    ctx = _prim_ctx(rho.shape, box_size, box_min)
    ctx.call("baorec_set_tune_binned", 0 if binned is None else int(bool(binned)))
    p = _Particles(x, y, z, w)
    flags = p.flags | (_lib.WRITEBACK if wrap else 0) | (_lib.DETERMINISTIC if deterministic else 0)
    with _Mesh(rho) as m:
        ctx.call(name, m.ptr, p.ptrs[0], p.ptrs[1], p.ptrs[2], p.ptrs[3], p.n, int(bool(wrap)), flags)
    if wrap:   # the reference writes the wrapped positions back into its inputs
        for i in range(3):
            p.writeback(i)
    return rho


def cic_(rho, x, y, z, w, box_size, box_min, wrap=True, deterministic=False, binned=None):
    """``cic!`` (``src/mas.jl:1-107``): add CIC weights to ``rho``.  ``binned``
    picks the FP32 paint (None / False: one float atomic per weight, as the
    reference's GPU kernel; True: tile counting sort and shared-memory tiles)."""
    return _paint("baorec_cic", rho, x, y, z, w, box_size, box_min, wrap, deterministic, binned)


def tsc_(rho, x, y, z, w, box_size, box_min, wrap=True, deterministic=False, binned=None):
    """Triangular-shaped-cloud paint (no reference counterpart); ``binned`` as
    for :func:`cic_`."""
    return _paint("baorec_tsc", rho, x, y, z, w, box_size, box_min, wrap, deterministic, binned)


def cell_bins(x, y, z, box_size, box_min, dims, wrap=True):
    """Lower CIC cell key per particle and the count per cell (int32),
    computed by the paint's own binning (integer, bit-exact)."""
    ctx = _prim_ctx(dims, box_size, box_min)
    p = _Particles(x, y, z)
    if p.device:
        torch = _torch()
        keys = torch.empty(p.n, dtype=torch.int32, device="cuda")
        counts = torch.empty(int(np.prod(dims)), dtype=torch.int32, device="cuda")
        _sync_torch()
        ctx.call("baorec_cell_bins", p.ptrs[0], p.ptrs[1], p.ptrs[2], p.n, int(bool(wrap)), 0,
                 keys.data_ptr(), counts.data_ptr())
        return keys, counts.reshape(dims[2], dims[1], dims[0]).permute(2, 1, 0)
    keys = np.empty(p.n, dtype=np.int32)
    counts = np.empty(int(np.prod(dims)), dtype=np.int32)
    ctx.call("baorec_cell_bins", p.ptrs[0], p.ptrs[1], p.ptrs[2], p.n, int(bool(wrap)), _lib.HOST,
             keys.ctypes.data, counts.ctypes.data)
    return keys, counts.reshape(dims, order="F")


def read_cic_(output, field, x, y, z, box_size, box_min, wrap=True):
    """``read_cic!`` (``src/mas.jl:218-327``): trilinear read at the particles."""
    if not wrap:
        raise NotImplementedError("read_cic! is only called with wrap=true by the reference")
    ctx = _prim_ctx(field.shape, box_size, box_min)
    p = _Particles(x, y, z)
    out = _Particles(output)
    if out.device != p.device:
        raise TypeError("output and positions must live on the same side")
    with _Mesh(field, write=False) as m:
        ctx.call("baorec_read_cic", m.ptr, p.ptrs[0], p.ptrs[1], p.ptrs[2], p.n, out.ptrs[0], p.flags)
    out.writeback(0)
    return output


# ----------------------------------------------------------------------------
# k-space and overdensity
# ----------------------------------------------------------------------------

def smooth_(field, smoothing_radius, box_size, fft_plan=None):
    """``smooth!`` (``src/utils.jl:45-96``)."""
    ctx = _prim_ctx(field.shape, box_size, [0.0, 0.0, 0.0], smoothing_radius=float(smoothing_radius))
    with _Mesh(field) as m:
        ctx.call("baorec_smooth", m.ptr)
    return field


def setup_overdensity_(delta, recon, x, y, z, w, rx=None, ry=None, rz=None, rw=None, wrap=True, ran_min=0.01):
    """``setup_overdensity!`` data only (``src/recon.jl:42-57``) or with
    randoms (``src/recon.jl:60-91``).  ``delta`` accumulates the paint (pass zeros)."""
    ctx = _ctx(recon, delta.shape, ran_min)
    if rx is None:
        p = _Particles(x, y, z, w)
        flags = p.flags | (_lib.WRITEBACK if wrap else 0) | _det(recon)
        with _Mesh(delta) as m:
            ctx.call("baorec_setup_overdensity", m.ptr, *p.ptrs, p.n, int(bool(wrap)), flags)
        if wrap:
            for i in range(3):
                p.writeback(i)
    else:
        p = _Particles(x, y, z, w, rx, ry, rz, rw)
        n = _Particles(x).n
        nr = _Particles(rx).n
        with _Mesh(delta) as m:
            ctx.call("baorec_setup_overdensity_randoms", m.ptr, *p.ptrs[:4], n, *p.ptrs[4:], nr, p.flags | _det(recon))
    return delta


def iterate_(delta_r, delta_s, it, recon):
    """``iterate!`` (``src/iterative.jl:5-211``) for the 1-based iteration ``it``."""
    ctx = _ctx(recon, delta_r.shape)
    with _Mesh(delta_r) as a, _Mesh(delta_s, write=False) as b:
        ctx.call("baorec_iterate", a.ptr, b.ptr, int(it))
    return delta_r


def _det(recon) -> int:
    return _lib.DETERMINISTIC if getattr(recon, "deterministic", False) else 0


def _catalog_call(name, recon, shape, x, y, z, w, randoms, writeback):
    ctx = _ctx(recon, shape)
    if randoms is None:
        p = _Particles(x, y, z, w)
        n, nr = p.n, 0
        rp = [None] * 4
    else:
        p = _Particles(x, y, z, w, *randoms)
        n = _Particles(x).n
        nr = _Particles(randoms[0]).n
        rp = p.ptrs[4:]
    flags = p.flags | (_lib.WRITEBACK if (writeback and randoms is None) else 0) | _det(recon)
    _sync_torch()
    st = ctx.status(name, *p.ptrs[:4], n, *rp, nr, flags)
    if st not in (_lib.OK, _lib.ERR_NOT_CONVERGED):
        _lib.check(ctx.h, st)
    if writeback and randoms is None:
        for i in range(3):
            p.writeback(i)
    bs, bm = ctx.box()
    recon.box_size = np.array(bs, dtype=F32)
    recon.box_min = np.array(bm, dtype=F32)
    if isinstance(recon, MultigridRecon) and recon.mg_mode == "convergent":
        recon.solve_stats = dict(ctx.solve_stats(), status=int(st))
    return ctx, p.device, st


def reconstructed_overdensity_(delta, recon, x, y, z, w, rx=None, ry=None, rz=None, rw=None):
    """``reconstructed_overdensity!`` (``src/recon.jl:93-132``)."""
    randoms = None if rx is None else (rx, ry, rz, rw)
    ctx, dev, _ = _catalog_call("baorec_reconstructed_overdensity", recon, delta.shape, x, y, z, w, randoms, True)
    res = _result_to(ctx, dev, delta.shape)
    if _is_torch(delta):
        delta.copy_(res)
    else:
        delta[...] = res
    return delta


def reconstructed_potential_(phi, recon, x, y, z, w, rx=None, ry=None, rz=None, rw=None):
    """``reconstructed_potential!`` (``src/recon.jl:184-212``)."""
    randoms = None if rx is None else (rx, ry, rz, rw)
    ctx, dev, st = _catalog_call("baorec_reconstructed_potential", recon, phi.shape, x, y, z, w, randoms, True)
    res = _result_to(ctx, dev, phi.shape)
    if _is_torch(phi):
        phi.copy_(res)
    else:
        phi[...] = res
    if st == _lib.ERR_NOT_CONVERGED:
        _lib.check(ctx.h, st)
    return phi


def run_(recon, grid_size, x, y, z, w, rx=None, ry=None, rz=None, rw=None):
    """``run!`` (``src/recon.jl:134-261``).  With randoms the box is replaced by
    ``setup_box(randoms, 500)``.  Sets ``recon.result_cache`` (host or device,
    like the inputs) and returns it."""
    randoms = None if rx is None else (rx, ry, rz, rw)
    if randoms is None and (recon.box_size is None or recon.box_min is None):
        raise ValueError("run! without randoms needs recon.box_size and recon.box_min")
    if recon.box_size is None:
        recon.box_size, recon.box_min = [1.0, 1.0, 1.0], [0.0, 0.0, 0.0]
    ctx, dev, st = _catalog_call("baorec_run", recon, tuple(grid_size), x, y, z, w, randoms, True)
    recon.result_cache = _result_to(ctx, dev, tuple(grid_size))
    if st == _lib.ERR_NOT_CONVERGED:
        _lib.check(ctx.h, st)
    return recon.result_cache


def _set_field(ctx, mesh):
    if _is_torch(mesh):
        with _Mesh(mesh, write=False) as m:
            ctx.call("baorec_set_result", m.ptr, 0)
    else:
        h = np.asfortranarray(mesh, dtype=F32)
        ctx.call("baorec_set_result", h.ctypes.data, _lib.HOST)


def _shifts(name, recon, x, y, z, mesh, field):
    if field not in _lib.FIELD:
        raise ValueError(f"field must be :disp, :rsd or :sum, got {field!r}")
    if mesh is None:
        mesh = recon.result_cache
        if mesh is None:
            raise BaorecError(_lib.ERR_STATE, "no reconstruction result (run! first)")
    ctx = _ctx(recon, mesh.shape)
    _set_field(ctx, mesh)
    p = _Particles(x, y, z)
    outs = [_vec_out(p.n, p.device) for _ in range(3)]
    _sync_torch()
    ctx.call(name, *p.ptrs, p.n, _lib.FIELD[field], *[_vptr(o) for o in outs], p.flags)
    return tuple(outs)


def read_shifts(recon, x, y, z, delta_r=None, field="disp"):
    """``read_shifts`` (``src/recon.jl:264-364``) → (sx, sy, sz)."""
    return _shifts("baorec_read_shifts", recon, x, y, z, delta_r, field)


def reconstructed_positions(recon, x, y, z, delta_r=None, field="disp"):
    """``reconstructed_positions`` (``src/recon.jl:366-388``) → new arrays p - shift."""
    return _shifts("baorec_reconstructed_positions", recon, x, y, z, delta_r, field)


def reconstructed_positions2(recon, x, y, z, delta_r=None, fields=("sum", "disp")):
    """Two ``reconstructed_positions`` of the same particles from one gather
    of the displacement (the examples' ``:sum`` and ``:disp`` randoms);
    returns (positions for fields[0], positions for fields[1]), each
    bit-identical to its single call."""
    for fl in fields:
        if fl not in _lib.FIELD:
            raise ValueError(f"field must be :disp, :rsd or :sum, got {fl!r}")
    mesh = delta_r if delta_r is not None else recon.result_cache
    if mesh is None:
        raise BaorecError(_lib.ERR_STATE, "no reconstruction result (run! first)")
    ctx = _ctx(recon, mesh.shape)
    _set_field(ctx, mesh)
    p = _Particles(x, y, z)
    a = [_vec_out(p.n, p.device) for _ in range(3)]
    b = [_vec_out(p.n, p.device) for _ in range(3)]
    _sync_torch()
    ctx.call("baorec_reconstructed_positions2", *p.ptrs, p.n, _lib.FIELD[fields[0]], *[_vptr(o) for o in a],
             _lib.FIELD[fields[1]], *[_vptr(o) for o in b], p.flags)
    return tuple(a), tuple(b)


def compute_displacements(field_mesh, recon):
    """The three displacement meshes of ``compute_displacements``
    (``src/iterative.jl:229-275`` / ``src/multigrid.jl:755-799``) as CUDA tensors."""
    ctx = _ctx(recon, field_mesh.shape)
    _set_field(ctx, field_mesh)
    outs = [zeros_mesh(field_mesh.shape) for _ in range(3)]
    _sync_torch()
    ctx.call("baorec_displacement_meshes", *[o.data_ptr() for o in outs])
    return tuple(outs)


# ----------------------------------------------------------------------------
# multigrid primitives — src/multigrid.jl
# ----------------------------------------------------------------------------

def _nl(shape):
    return (C.c_int32 * 3)(*[int(s) for s in shape])


def _mg_ctx(recon, top_shape):
    if not isinstance(recon, MultigridRecon):
        raise TypeError("multigrid primitives need a MultigridRecon")
    return _ctx(recon, top_shape)


def jacobi_(v, f, recon, niterations, top_shape=None):
    """``jacobi!`` (``src/multigrid.jl:14-210``) on a level of the recon mesh."""
    ctx = _mg_ctx(recon, top_shape or v.shape)
    with _Mesh(v) as a, _Mesh(f, write=False) as b:
        ctx.call("baorec_mg_jacobi", a.ptr, b.ptr, _nl(v.shape), int(niterations))
    return v


def residual_(r, v, f, recon, top_shape=None):
    """``residual!`` (``src/multigrid.jl:213-395``): r = f - A v."""
    ctx = _mg_ctx(recon, top_shape or v.shape)
    with _Mesh(r) as a, _Mesh(v, write=False) as b, _Mesh(f, write=False) as c:
        ctx.call("baorec_mg_residual", a.ptr, b.ptr, c.ptr, _nl(v.shape))
    return r


def reduce_(v2h, v1h, recon, top_shape=None):
    """``reduce!`` (``src/multigrid.jl:520-651``): restriction v1h → v2h."""
    ctx = _mg_ctx(recon, top_shape or v1h.shape)
    with _Mesh(v2h) as a, _Mesh(v1h, write=False) as b:
        ctx.call("baorec_mg_reduce", a.ptr, b.ptr, _nl(v1h.shape))
    return v2h


def prolong_(v1h, v2h, recon, top_shape=None):
    """``prolong!`` (``src/multigrid.jl:398-518``): prolongation v2h → v1h (overwrites)."""
    ctx = _mg_ctx(recon, top_shape or v1h.shape)
    with _Mesh(v1h) as a, _Mesh(v2h, write=False) as b:
        ctx.call("baorec_mg_prolong", a.ptr, b.ptr, _nl(v1h.shape))
    return v1h


def vcycle_(v, f, recon, top_shape=None):
    """``vcycle!`` (``src/multigrid.jl:654-719``)."""
    ctx = _mg_ctx(recon, top_shape or v.shape)
    with _Mesh(v) as a, _Mesh(f, write=False) as b:
        ctx.call("baorec_mg_vcycle", a.ptr, b.ptr, _nl(v.shape))
    return v


def fmg(f1h, v1h, recon):
    """``fmg`` (``src/multigrid.jl:722-752``): returns the FMG solution (written to v1h)."""
    ctx = _mg_ctx(recon, f1h.shape)
    if v1h is None:
        v1h = _empty_like_kind(f1h.shape, _is_torch(f1h))
    with _Mesh(v1h) as a, _Mesh(f1h, write=False) as b:
        ctx.call("baorec_mg_fmg", b.ptr, a.ptr)
    return v1h


def solve_(phi, f, recon, phi0=None):
    """Residual-driven multigrid solve (no reference counterpart): V-cycles
    until ``|f - α - A φ| <= rtol |f - α|``.  Returns the stats dict."""
    ctx = _mg_ctx(recon, f.shape)
    st = _lib.SolveStats()
    with _Mesh(phi) as a, _Mesh(f, write=False) as b:
        if phi0 is not None:
            with _Mesh(phi0, write=False) as c:
                code = ctx.status("baorec_mg_solve", b.ptr, a.ptr, c.ptr, C.byref(st))
        else:
            code = ctx.status("baorec_mg_solve", b.ptr, a.ptr, None, C.byref(st))
    stats = dict(st.as_dict(), status=code)
    recon.solve_stats = stats
    if code != _lib.OK:
        _lib.check(ctx.h, code)
    return stats
