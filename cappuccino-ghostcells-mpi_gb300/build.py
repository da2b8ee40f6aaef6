"""Build the native library libcappgpu.so for sm_103a with nvcc.

Translation units are compiled in parallel and linked into one shared
library in <package>/_build/.  FP64 kernels are compiled with --fmad=false:
the reference (gfortran -O2, x86-64) rounds every multiply and add
separately, and bit-identical results need the same.
"""
import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libcappgpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC",
              "-I" + str(ROOT / "include")]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def sources():
    return sorted(CSRC.glob("*.cu"))


def _stale():
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [ROOT / "include" / "cappgpu.h", pathlib.Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force=False, verbose=False, jobs=None):
    """Compile every .cu under csrc/ and link libcappgpu.so; returns its path.
    Extra nvcc flags (e.g. -D overrides of tuning constants) may be given in
    the environment variable CAPPGPU_NVCC_FLAGS."""
    extra = os.environ.get("CAPPGPU_NVCC_FLAGS", "").split()
    if not force and not extra and not _stale():
        return LIB
    OUT.mkdir(exist_ok=True)
    exe = nvcc()
    srcs = sources()

    def compile_one(src):
        obj = OUT / (src.stem + ".o")
        cmd = [exe, *ARCH, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = OUT / "libcappgpu.so.tmp"
    cudalib = pathlib.Path(exe).resolve().parent.parent / "lib64"
    cmd = [exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart",
           "-Xlinker", "-rpath", "-Xlinker", str(cudalib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="-f" in sys.argv, verbose=True))
