"""ctypes binding of libbaorec_gb300.so (the C ABI in include/baorec_gb300.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

OK = 0
ERR_ARG, ERR_CUDA, ERR_CUFFT, ERR_NOT_CONVERGED, ERR_OOB, ERR_STATE, ERR_NOMEM = 1, 2, 3, 4, 5, 6, 7
ERR_TOO_LARGE = 8
HOST, ASYNC, WRITEBACK, DETERMINISTIC = 0x1, 0x2, 0x4, 0x8
ITERATIVE, MULTIGRID = 0, 1
LOS_LOCAL, LOS_GLOBAL = 0, 1
MAS_CIC, MAS_TSC = 0, 1
MG_REFERENCE, MG_CONVERGENT = 0, 1
START_ZERO, START_SPECTRAL, START_LEARNED = 0, 1, 2
FIELD = {"disp": 0, "rsd": 1, "sum": 2}


class BaorecError(RuntimeError):
    """A non-zero status from the library (message from baorec_last_error)."""

    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class BoundsError(BaorecError, IndexError):
    """Particle outside the mesh; the reference raises Julia's BoundsError."""


class NotConverged(BaorecError):
    """The residual-driven multigrid solve hit its cycle cap."""


class Config(C.Structure):
    _fields_ = [
        ("method", C.c_int32), ("n", C.c_int32 * 3), ("box_size", C.c_float * 3), ("box_min", C.c_float * 3),
        ("los_mode", C.c_int32), ("los", C.c_float * 3), ("bias", C.c_float), ("f", C.c_float),
        ("smoothing_radius", C.c_float), ("beta", C.c_float), ("n_iter", C.c_int32),
        ("jacobi_damping_factor", C.c_float), ("jacobi_niterations", C.c_int32),
        ("vcycle_niterations", C.c_int32), ("ran_min", C.c_float), ("mas", C.c_int32),
        ("mg_mode", C.c_int32), ("nu1", C.c_int32), ("nu2", C.c_int32), ("rtol", C.c_float),
        ("max_cycles", C.c_int32), ("mg_start", C.c_int32), ("start_rate", C.c_float),
    ]


class GuessTrainConfig(C.Structure):
    _fields_ = [("steps", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("seed", C.c_uint32),
                ("sigma_g", C.c_float), ("pk_slope", C.c_float), ("region_min", C.c_float * 3),
                ("region_size", C.c_float * 3), ("r_min", C.c_float), ("r_max", C.c_float),
                ("ra_min", C.c_float), ("ra_max", C.c_float), ("dec_min", C.c_float), ("dec_max", C.c_float),
                ("rtol", C.c_float), ("loss", C.c_int32)]


class PowerConfig(C.Structure):
    _fields_ = [("geometry", C.c_int32), ("mas", C.c_int32), ("interlace", C.c_int32), ("nbins", C.c_int32),
                ("kmin", C.c_float), ("dk", C.c_float), ("los", C.c_float * 3), ("reserved", C.c_int32)]


POWER_BOX, POWER_SURVEY = 0, 1


class BatchItem(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p), ("w", C.c_void_p), ("n", C.c_int64),
                ("mesh", C.c_int32), ("box_size", C.c_float), ("mas", C.c_int32), ("smoothing_radius", C.c_float),
                ("field", C.c_int32), ("out_x", C.c_void_p), ("out_y", C.c_void_p), ("out_z", C.c_void_p)]


class SolveStats(C.Structure):
    _fields_ = [("cycles", C.c_int32), ("spectral_steps", C.c_int32), ("rel_residual", C.c_double), ("alpha", C.c_double),
                ("rel_residual_initial", C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


P = C.c_void_p
I64 = C.c_int64
U32 = C.c_uint32
I32P = C.POINTER(C.c_int32)
F3 = C.c_float * 3

_SIGS = {
    "baorec_config_default": (None, [C.POINTER(Config)]),
    "baorec_create": (C.c_int, [C.POINTER(Config), C.POINTER(P)]),
    "baorec_destroy": (C.c_int, [P]),
    "baorec_last_error": (C.c_char_p, [P]),
    "baorec_set_box": (C.c_int, [P, F3, F3]),
    "baorec_get_box": (C.c_int, [P, F3, F3]),
    "baorec_stream": (P, [P]),
    "baorec_kernel_launches": (I64, [P]),
    "baorec_total_kernel_launches": (I64, []),
    "baorec_result_ptr": (P, [P]),
    "baorec_setup_box": (C.c_int, [P, P, P, P, I64, C.c_float, U32, F3, F3]),
    "baorec_setup_box_noalloc": (C.c_int, [P, P, P, I64, C.c_float, P, F3, F3]),
    "baorec_cic": (C.c_int, [P, P, P, P, P, P, I64, C.c_int, U32]),
    "baorec_tsc": (C.c_int, [P, P, P, P, P, P, I64, C.c_int, U32]),
    "baorec_cell_bins": (C.c_int, [P, P, P, P, I64, C.c_int, U32, P, P]),
    "baorec_smooth": (C.c_int, [P, P]),
    "baorec_setup_overdensity": (C.c_int, [P, P, P, P, P, P, I64, C.c_int, U32]),
    "baorec_setup_overdensity_randoms": (C.c_int, [P, P, P, P, P, P, I64, P, P, P, P, I64, U32]),
    "baorec_iterate": (C.c_int, [P, P, P, C.c_int]),
    "baorec_mg_jacobi": (C.c_int, [P, P, P, I32P, C.c_int]),
    "baorec_mg_residual": (C.c_int, [P, P, P, P, I32P]),
    "baorec_mg_reduce": (C.c_int, [P, P, P, I32P]),
    "baorec_mg_prolong": (C.c_int, [P, P, P, I32P]),
    "baorec_mg_vcycle": (C.c_int, [P, P, P, I32P]),
    "baorec_mg_fmg": (C.c_int, [P, P, P]),
    "baorec_mg_solve": (C.c_int, [P, P, P, P, C.POINTER(SolveStats)]),
    "baorec_last_solve_stats": (C.c_int, [P, C.POINTER(SolveStats)]),
    "baorec_solve_history": (C.c_int, [P, C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_int]),
    "baorec_start_residual": (C.c_int, [P, P, C.c_int, C.POINTER(C.c_double)]),
    "baorec_fft_callbacks": (C.c_int, [P, C.POINTER(C.c_char_p)]),
    "baorec_set_fft_callbacks": (C.c_int, [P, C.c_int]),
    "baorec_profile_kernel": (C.c_int, [P, C.c_int, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "baorec_reconstructed_overdensity": (C.c_int, [P, P, P, P, P, I64, P, P, P, P, I64, U32]),
    "baorec_reconstructed_potential": (C.c_int, [P, P, P, P, P, I64, P, P, P, P, I64, U32]),
    "baorec_run": (C.c_int, [P, P, P, P, P, I64, P, P, P, P, I64, U32]),
    "baorec_get_result": (C.c_int, [P, P, U32]),
    "baorec_set_result": (C.c_int, [P, P, U32]),
    "baorec_displacement_meshes": (C.c_int, [P, P, P, P]),
    "baorec_batch_create": (C.c_int, [C.POINTER(Config), C.POINTER(BatchItem), C.c_int, C.POINTER(P)]),
    "baorec_batch_launch": (C.c_int, [P, P]),
    "baorec_batch_sync": (C.c_int, [P, P]),
    "baorec_batch_stream": (P, [P]),
    "baorec_batch_kernel_launches": (I64, [P]),
    "baorec_batch_last_error": (C.c_char_p, [P]),
    "baorec_batch_destroy": (C.c_int, [P]),
    "baorec_autotune": (C.c_int, [P, U32, I32P, I32P]),
    "baorec_set_tune": (C.c_int, [P, C.c_int32, I32P]),
    "baorec_tune_stream": (C.c_int, [P]),
    "baorec_set_tune_stream": (C.c_int, [P, C.c_int]),
    "baorec_tune_pairs": (C.c_int, [P]),
    "baorec_set_tune_pairs": (C.c_int, [P, C.c_int]),
    "baorec_tune_binned": (C.c_int, [P]),
    "baorec_set_tune_binned": (C.c_int, [P, C.c_int]),
    "baorec_tune_acc": (C.c_int, [P]),
    "baorec_set_tune_acc": (C.c_int, [P, C.c_int]),
    "baorec_tune_zpass": (C.c_int, [P]),
    "baorec_set_tune_zpass": (C.c_int, [P, C.c_int]),
    "baorec_tune_xy": (C.c_int, [P]),
    "baorec_set_tune_xy": (C.c_int, [P, C.c_int]),
    "baorec_sky_to_cartesian": (C.c_int, [P, P, P, P, I64, P, C.c_int32, C.c_double, C.c_double, C.c_float,
                                          P, P, P, U32]),
    "baorec_cartesian_to_sky": (C.c_int, [P, P, P, P, I64, P, C.c_int32, C.c_double, C.c_double, C.c_float,
                                          P, P, P, U32]),
    "baorec_fkp_weights": (C.c_int, [P, P, I64, C.c_float, P, U32]),
    "baorec_guess_num_params": (I64, []),
    "baorec_guess_init": (C.c_int, [P, C.c_uint32]),
    "baorec_guess_set_params": (C.c_int, [P, P, I64]),
    "baorec_guess_get_params": (C.c_int, [P, P, I64]),
    "baorec_guess_eval": (C.c_int, [P, P, P, P, P, C.POINTER(C.c_double), C.c_int]),
    "baorec_guess_apply": (C.c_int, [P, P, P]),
    "baorec_guess_set_level": (C.c_int, [P, C.c_int32]),
    "baorec_guess_level": (C.c_int32, [P]),
    "baorec_guess_sample": (C.c_int, [P, C.POINTER(GuessTrainConfig), I64, P, P]),
    "baorec_guess_train": (C.c_int, [P, C.POINTER(GuessTrainConfig), P]),
    "baorec_set_gradient": (C.c_int, [P, C.c_int32]),
    "baorec_reconstructed_positions2": (C.c_int, [P, P, P, P, I64, C.c_int, P, P, P, C.c_int, P, P, P, C.c_uint32]),
    "baorec_read_ascii": (C.c_int, [P, C.c_char_p, P, C.c_int32, C.c_int32, C.c_int32, P, I64,
                                    C.POINTER(C.c_int64), C.c_uint32]),
    "baorec_write_npy": (C.c_int, [P, C.c_char_p, P, C.c_int32, I64, C.c_uint32]),
    "baorec_power_multipoles": (C.c_int, [P, C.POINTER(PowerConfig), P, P, P, P, I64, P, P, P, P, P, I64,
                                          P, P, P, P, P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_uint32]),
    "baorec_guess_set_conv_path": (C.c_int, [P, C.c_int32]),
    "baorec_guess_tc_layers": (C.c_int32, [P]),
    "baorec_guess_conv3": (C.c_int, [P, C.c_int32, C.c_int32, C.c_int32, P, P, P, P, P, C.c_int32, C.c_int32]),
    "baorec_guess_conv3_held_back": (C.c_int, [P, C.c_int32, C.c_int32, C.c_int32, C.c_int64]),
    "baorec_guess_profile_conv": (C.c_int, [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                            C.POINTER(C.c_float), C.POINTER(C.c_double)]),
    "baorec_read_cic": (C.c_int, [P, P, P, P, P, I64, P, U32]),
    "baorec_read_shifts": (C.c_int, [P, P, P, P, I64, C.c_int, P, P, P, U32]),
    "baorec_reconstructed_positions": (C.c_int, [P, P, P, P, I64, C.c_int, P, P, P, U32]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load the shared library (building it first when it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(f"libbaorec_gb300.so not built ({path}); run __graft_entry__.build()")
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGS)


def check(ctx, status):
    if status == OK:
        return
    msg = load().baorec_last_error(ctx)
    msg = msg.decode() if msg else ""
    if status == ERR_OOB:
        raise BoundsError(status, msg)
    if status == ERR_NOT_CONVERGED:
        raise NotConverged(status, msg)
    raise BaorecError(status, msg)


def default_config() -> Config:
    c = Config()
    load().baorec_config_default(C.byref(c))
    return c


class Context:
    """Owns one baorec_ctx (mesh buffers, cuFFT plans, stream)."""

    def __init__(self, cfg: Config):
        self.lib = load()
        h = P()
        st = self.lib.baorec_create(C.byref(cfg), C.byref(h))
        if st != OK:
            msg = self.lib.baorec_last_error(None)
            raise BaorecError(st, msg.decode() if msg else "create failed")
        self.h = h
        self.cfg = cfg

    def close(self):
        if getattr(self, "h", None):
            self.lib.baorec_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def call(self, name, *args):
        check(self.h, getattr(self.lib, name)(self.h, *args))

    def status(self, name, *args):
        """Call and return the raw status (for NOT_CONVERGED handling)."""
        return getattr(self.lib, name)(self.h, *args)

    @property
    def stream(self) -> int:
        return self.lib.baorec_stream(self.h) or 0

    def launches(self) -> int:
        return int(self.lib.baorec_kernel_launches(self.h))

    def total_launches(self) -> int:
        """This library's kernel launches in the process so far (every context)."""
        return int(self.lib.baorec_total_kernel_launches())

    def box(self):
        bs, bm = F3(), F3()
        self.call("baorec_get_box", bs, bm)
        return list(bs), list(bm)

    def solve_stats(self) -> dict:
        st = SolveStats()
        self.call("baorec_last_solve_stats", C.byref(st))
        return st.as_dict()

    def autotune(self, stencil: bool = True, paint: bool = True) -> dict:
        """Pick launch shapes by timing (baorec_autotune); returns the choices."""
        pt = C.c_int32()
        bt = (C.c_int32 * 16)()
        self.call("baorec_autotune", (1 if stencil else 0) | (2 if paint else 0), C.byref(pt), bt)
        return {"paint_tile": pt.value, "paint_binned": int(self.lib.baorec_tune_binned(self.h)),
                "tile16_per_level": list(bt),
                "stream_residuals": int(self.lib.baorec_tune_stream(self.h)),
                "pair_residual": int(self.lib.baorec_tune_pairs(self.h)),
                "acc_residual": int(self.lib.baorec_tune_acc(self.h)),
                "fft_zpass": int(self.lib.baorec_tune_zpass(self.h)),
                "fft_xy_fused": int(self.lib.baorec_tune_xy(self.h))}

    def fft_callbacks(self) -> dict:
        """State of the FFT start's cuFFT load callback (baorec_fft_callbacks)."""
        note = C.c_char_p()
        st = self.lib.baorec_fft_callbacks(self.h, C.byref(note))
        return {"state": int(st), "note": (note.value or b"").decode()}

    def solve_history(self) -> list:
        """[(relative residual, correction that followed)] of the last solve:
        0 = V-cycle, m > 0 = m FFT corrections, -1 = none."""
        n = self.lib.baorec_solve_history(self.h, None, None, 0)
        if n < 0:
            raise BaorecError(-n, "solve_history")
        rho = (C.c_double * max(n, 1))()
        kind = (C.c_int32 * max(n, 1))()
        self.lib.baorec_solve_history(self.h, rho, kind, n)
        return [(rho[i], kind[i]) for i in range(n)]

    def set_box(self, box_size, box_min):
        self.call("baorec_set_box", F3(*box_size), F3(*box_min))
