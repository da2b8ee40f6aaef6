"""cappgpu_spmv_noalloc (fixed device scratch, no allocation) against
cappgpu_spmv, called through the C ABI.  Kept in its own file, named to be
collected last; it passes alone in a fresh process as well."""
import ctypes

import numpy as np
import pytest

import cappgpu


def fid(name):
    return cappgpu.FIELD[name]

pytestmark = pytest.mark.gpu


def _random_system(lib, ni, nj, nk, seed):
    lib.init(ni, nj, nk)
    n = ni * nj * nk
    rng = np.random.default_rng(seed)
    off = {f: rng.uniform(0.05, 1.0, n) for f in ("ae", "aw", "an", "as", "at", "ab")}
    for f, a in off.items():
        lib.set_field(f, a)
    lib.set_field("ap", sum(off.values()) * 1.5)
    lib.set_field("u", rng.uniform(-1.0, 1.0, n))   # ghost layers included: the stencil reads them


def _call(lib, name, pk, zk):
    dot = ctypes.c_double(np.nan)
    rc = getattr(lib.lib, name)(fid(pk), fid(zk), ctypes.byref(dot))
    assert rc == 0, lib.lib.cappgpu_last_error().decode()
    return dot.value, lib.get_field(zk)


@pytest.mark.parametrize("dims", [(14, 13, 12), (68, 37, 45)])
def test_noalloc_matches_spmv_twice(gpu_lib, dims):
    _random_system(gpu_lib, *dims, seed=7)
    d_ref, z_ref = _call(gpu_lib, "cappgpu_spmv", "u", "pp")
    for _ in range(2):   # two calls in a row: the scratch needs no reset between calls
        gpu_lib.set_field("pp", np.zeros(gpu_lib.nijk))
        d, z = _call(gpu_lib, "cappgpu_spmv_noalloc", "u", "pp")
        assert np.array_equal(z, z_ref)                      # same per-cell arithmetic
        assert abs(d - d_ref) <= 1e-12 * abs(d_ref)           # other fixed summation order


def test_noalloc_rejects_grid_beyond_scratch(gpu_lib):
    gpu_lib.init(208, 208, 199)   # 204 x 204 x 195 = 8,115,120 interior cells: fits
    dot = ctypes.c_double()
    assert gpu_lib.lib.cappgpu_spmv_noalloc(fid("u"), fid("pp"), ctypes.byref(dot)) == 0
    gpu_lib.init(210, 210, 204)   # 206 x 206 x 200 = 8,487,200 interior cells: beyond 8,388,608
    rc = gpu_lib.lib.cappgpu_spmv_noalloc(fid("u"), fid("pp"), ctypes.byref(dot))
    assert rc == -2   # CAPPGPU_E_ARG
    assert b"fixed scratch" in gpu_lib.lib.cappgpu_last_error()
