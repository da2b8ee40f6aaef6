"""Import shim for the package directory ``cappuccino-ghostcells-mpi_gb300/``.

The directory name contains hyphens, which Python cannot import by name;
``import cappgpu`` loads it as the package ``cappgpu``.
"""
import importlib.util
import pathlib
import sys

_DIR = pathlib.Path(__file__).resolve().parent / "cappuccino-ghostcells-mpi_gb300"

if "cappgpu._pkg" not in sys.modules:
    _spec = importlib.util.spec_from_file_location(
        "cappgpu._pkg", _DIR / "__init__.py", submodule_search_locations=[str(_DIR)])
    _pkg = importlib.util.module_from_spec(_spec)
    sys.modules["cappgpu._pkg"] = _pkg
    _spec.loader.exec_module(_pkg)
_pkg = sys.modules["cappgpu._pkg"]

params = _pkg.params
cases = _pkg.cases
fortio = _pkg.fortio
build = _pkg.build
Library = _pkg.Library
CappError = _pkg.CappError
load_library = _pkg.load_library
SIGNATURES = _pkg.SIGNATURES
FIELD = _pkg.FIELD
FIELD_NAMES = _pkg.FIELD_NAMES
Params = _pkg.Params
SolveReport = _pkg.SolveReport
SOLVER = _pkg.SOLVER
PACKAGE_DIR = _DIR
