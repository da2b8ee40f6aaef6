"""GB300 (sm_103a) implementation of Cappuccino's SIMPLE/PISO step on a
structured single-block ghost-cell grid (reference:
kiranhegde/cappuccino-ghostcells-mpi).

Layout:
  csrc/      CUDA kernels and the C ABI (include/cappgpu.h) -> libcappgpu.so
  build.py   nvcc build of libcappgpu.so for sm_103a
  native.py  ctypes binding mirroring the reference routine interface
  params.py  ctypes mirrors of the ABI structures, field/BC identifiers
  cases.py   seeded synthetic grids and cases of the benchmarked shapes
  fortio.py  the reference's grid and restart file formats
"""
from . import params, cases, fortio  # noqa: F401
from .params import FIELD, FIELD_NAMES, BC_NAMES, Params, SolveReport, SOLVER  # noqa: F401
from .build import build, LIB  # noqa: F401
from .native import Library, CappError, load_library, SIGNATURES  # noqa: F401
