"""GB300-native BAO reconstruction with BAOrec.jl's API (Python host side).

``import baorec`` exposes the reference's reconstruction types and calls —
``IterativeRecon``, ``MultigridRecon``, ``run_`` (``run!``),
``reconstructed_positions``, ``read_shifts`` and the lower-level
``setup_overdensity_``, ``cic_``, ``smooth_``, ``iterate_``, ``fmg`` … — backed
by the CUDA library ``libbaorec_gb300.so`` (C ABI: ``include/baorec_gb300.h``).
"""
from .recon import *  # noqa: F401,F403
from .recon import __all__ as _recon_all
from . import mocks  # noqa: F401
from . import guess  # noqa: F401
from . import cosmo  # noqa: F401
from . import power  # noqa: F401
from . import catalog  # noqa: F401
from .batch import Batch  # noqa: F401
from ._lib import load as load_library, lib_path  # noqa: F401

__all__ = list(_recon_all) + ["mocks", "guess", "cosmo", "power", "catalog", "Batch", "load_library", "lib_path"]
