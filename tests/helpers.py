"""Test helpers: seeded states, copying a host (oracle) state to the GPU
context, and element-wise comparison of every module array."""
import numpy as np

import cappgpu
from cappgpu import FIELD_NAMES

GEOMETRY = ["x", "y", "z", "xc", "yc", "zc", "vol", "fx", "fy", "fz", "ar1x", "ar1y", "ar1z",
            "ar2x", "ar2y", "ar2z", "ar3x", "ar3y", "ar3z", "walldist"]
STATE = [n for n in FIELD_NAMES if n not in GEOMETRY]


def with_fluxes(case, st):
    """Initial face fluxes from the oracle's geometry (the library derives
    them from its own, bit-identical, geometry)."""
    for n in ("ar1x", "ar1y", "ar1z", "ar2x", "ar2y", "ar2z", "ar3x", "ar3y", "ar3z", "fx", "fy", "fz"):
        case.fields[n] = st.field(n).copy()
    if case.name in ("channel", "rans_channel"):
        fl = cappgpu.cases.initial_face_fluxes(case)
        for n, a in fl.items():
            case.fields[n] = a
            st.set_field(n, a)
    return case


def randomize(st, rng, names, lo=-1.0, hi=1.0):
    """Fill whole arrays (ghost and padding cells included) with seeded
    uniform values, so that stale-ghost reads of the reference are
    exercised."""
    for n in names:
        st.set_field(n, rng.uniform(lo, hi, st.nijk))


def diag_dominant_matrix(st, rng, margin=0.5, symmetric=False):
    """Seeded 7-diagonal matrix with positive off-diagonals and a dominant
    diagonal over the whole array, plus random su.  symmetric=True sets
    aw(i+1)=ae(i), as(j+1)=an(j), ab(k+1)=at(k) as the pressure equation
    has them."""
    off = {n: rng.uniform(0.05, 1.0, st.nijk) for n in ("ae", "aw", "an", "as", "at", "ab")}
    if symmetric:
        ni, nj, nk = st.dims
        v = lambda a: a.reshape(nk, ni, nj)
        v(off["aw"])[:, 1:, :] = v(off["ae"])[:, :-1, :]
        v(off["as"])[:, :, 1:] = v(off["an"])[:, :, :-1]
        v(off["ab"])[1:] = v(off["at"])[:-1]
    for n, a in off.items():
        st.set_field(n, a)
    st.set_field("ap", sum(off.values()) * (1.0 + margin))
    st.set_field("su", rng.uniform(-1, 1, st.nijk))


def push(lib, st):
    """Create the GPU context with exactly the oracle state's arrays."""
    ni, nj, nk = st.dims
    lib.init(ni, nj, nk)
    for n in FIELD_NAMES:
        lib.set_field(n, st.field(n))
    for face in cappgpu.params.BC_NAMES:
        lib.set_bc(face, st.bc(face))
    p = cappgpu.Params()
    ctypes_copy(p, st.params)
    lib.set_params(p)


def ctypes_copy(dst, src):
    import ctypes
    ctypes.memmove(ctypes.addressof(dst), ctypes.addressof(src), ctypes.sizeof(dst))


def compare(lib, st, exact=(), rtol=None, names=None, atol_scale=0.0):
    """Return {name: (max_abs_diff, rel_l2)} and assert: names in `exact`
    must match bit for bit (-0.0 == 0.0), the rest (when rtol is set)
    within rtol relative L2."""
    out = {}
    for n in (names or FIELD_NAMES):
        g = lib.get_field(n)
        o = st.field(n)
        diff = np.abs(g - o)
        nrm = np.linalg.norm(o)
        rel = np.linalg.norm(g - o) / nrm if nrm > 0 else np.linalg.norm(g - o)
        out[n] = (float(diff.max()), float(rel))
        if n in exact:
            bad = np.flatnonzero(g != o)
            assert bad.size == 0, (f"{n}: {bad.size} elements differ, first at {bad[:5]}: "
                                   f"gpu {g[bad[:3]]} oracle {o[bad[:3]]}")
        elif rtol is not None:
            assert np.all(np.isfinite(g)) == np.all(np.isfinite(o)), f"{n}: finiteness differs"
            assert rel <= rtol, f"{n}: relative L2 {rel:.3e} > {rtol:.1e} (max abs {diff.max():.3e})"
    return out
