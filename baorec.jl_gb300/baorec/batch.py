"""Batched periodic-box reconstructions replayed as one CUDA graph (no
reference counterpart): ``baorec_batch_*`` in include/baorec_gb300.h.

    b = Batch(IterativeRecon(bias=2.0, f=0.8, smoothing_radius=15.0, los=[0, 0, 1]),
              [dict(x=x, y=y, z=z, w=w, mesh=128, box_size=1000.0, mas="tsc",
                    smoothing_radius=12.0, field="sum", out=(ox, oy, oz)), ...])
    b.launch(); b.sync()           # every mock reconstructed; outputs in `out`

Arrays are CUDA tensors (float32, contiguous); they must stay alive and at
the same addresses for the life of the batch.
"""
from __future__ import annotations

import ctypes as C

from . import _lib
from .recon import _config

_MAS = {"cic": _lib.MAS_CIC, "tsc": _lib.MAS_TSC}


class Batch:
    def __init__(self, recon, items):
        self.lib = _lib.load()
        first = items[0]["mesh"]
        base = _config(recon, (first, first, first))
        self._keep = []
        arr = (_lib.BatchItem * len(items))()
        for i, it in enumerate(items):
            ox, oy, oz = it["out"]
            ts = (it["x"], it["y"], it["z"], it["w"], ox, oy, oz)
            for t in ts:
                if not (t.is_cuda and t.is_contiguous()):
                    raise ValueError("batch arrays must be contiguous CUDA tensors")
            self._keep.append(ts)
            a = arr[i]
            a.x, a.y, a.z, a.w = (t.data_ptr() for t in ts[:4])
            a.n = int(it["x"].numel())
            a.mesh = int(it["mesh"])
            a.box_size = float(it["box_size"])
            a.mas = _MAS[it.get("mas", "cic")]
            a.smoothing_radius = float(it.get("smoothing_radius", recon.smoothing_radius))
            a.field = _lib.FIELD[it.get("field", "sum")]
            a.out_x, a.out_y, a.out_z = ox.data_ptr(), oy.data_ptr(), oz.data_ptr()
        self._items = arr
        h = C.c_void_p()
        st = self.lib.baorec_batch_create(C.byref(base), arr, len(items), C.byref(h))
        self.h = h
        if st != _lib.OK:
            msg = self.lib.baorec_batch_last_error(h).decode()
            self.close()
            raise _lib.BaorecError(st, msg)

    def _check(self, st):
        if st != _lib.OK:
            raise _lib.BaorecError(st, self.lib.baorec_batch_last_error(self.h).decode())

    def launch(self, stream: int = 0):
        """Replay the batch on `stream` (a cudaStream_t handle, e.g.
        torch.cuda.current_stream().cuda_stream; 0 = the batch's own)."""
        self._check(self.lib.baorec_batch_launch(self.h, stream or None))

    def sync(self, stream: int = 0):
        self._check(self.lib.baorec_batch_sync(self.h, stream or None))

    @property
    def stream(self) -> int:
        return self.lib.baorec_batch_stream(self.h) or 0

    def kernel_launches(self) -> int:
        return int(self.lib.baorec_batch_kernel_launches(self.h))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.lib.baorec_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
