"""GB300 (sm_103a) FUNWAVE-TVD SSP-RK3 solver stage: Python host layer.

The compute path is the C-ABI library ``libfunwave_gpu.so`` built from
``csrc/`` (CUDA kernels + host API, declared in ``include/funwave_gpu.h``).
This package only builds it and drives it through ``ctypes``; it has no
compute fallback: constructing a :class:`Solver` fails loudly when the
library or a GPU is missing.

Layout of the Python side:
  ``params``  input.txt keys of the hot path with the reference's defaults
              (src/io.F) and a reader for input.txt files (mod_input.F)
  ``cases``   seeded synthetic cases (bathymetries, wavemakers)
  ``solver``  the ctypes binding and the :class:`Solver` object
  ``ensemble`` independent runs of uneven size stepped concurrently
  ``learned`` the learned coarse-grid correction (network, pairs, training)
"""
from .params import PARAM_DEFAULTS, read_input_txt, with_defaults  # noqa: F401
from .solver import (  # noqa: F401
    FW_ERRORS, FwError, Solver, build, lib_path, load_library, declared_symbols)
from . import cases  # noqa: F401
from .ensemble import Ensemble, max_runup  # noqa: F401
from . import learned  # noqa: F401
