"""In-tree build of the native library ``liblmg_gb300.so`` for sm_103a.

Translation units are compiled in parallel with nvcc (device code, one
``-gencode`` for sm_103a) and g++ (host-only C++), then linked with the static
CUDA runtime.  Objects go to ``libmobility_gb300/_build/``; the library sits
next to this file.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "liblmg_gb300.so"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra defines, object name)
UNITS = [
    ("mdot_launch.cu", ["-DLMG_REAL=float"], "mdot_f.o"),
    ("mdot_launch.cu", ["-DLMG_REAL=double"], "mdot_d.o"),
    ("solver.cu", [], "solver.o"),
    ("mdot_sym.cu", [], "mdot_sym.o"),
    ("probes.cu", [], "probes.o"),
    ("noalloc.cu", [], "noalloc.o"),
    ("precond.cu", [], "precond.o"),
    ("tc_gemm.cu", [], "tc_gemm.o"),
    ("ensemble.cu", [], "ensemble.o"),
    ("solver_base.cpp", [], "solver_base.o"),
    ("capi.cpp", [], "capi.o"),
    ("self_mobility.cpp", [], "self_mobility.o"),
]


def _nvcc():
    return shutil.which("nvcc") or str(CUDA_HOME / "bin" / "nvcc")


def _headers():
    return list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + list((ROOT / "include").glob("*.h"))


def _compile(src, defs, obj, objdir=None):
    s = CSRC / src
    o = (objdir or OBJ) / obj
    deps = [s] + _headers()
    if o.exists() and all(d.stat().st_mtime <= o.stat().st_mtime for d in deps):
        return None
    inc = [f"-I{ROOT / 'include'}", f"-I{CSRC}"]
    if src.endswith(".cu"):
        cmd = [_nvcc(), "-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
               "--expt-relaxed-constexpr", *defs, *inc, "-c", str(s), "-o", str(o)]
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", f"-I{CUDA_HOME / 'include'}", *defs, *inc,
               "-c", str(s), "-o", str(o)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
    return None


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> Path:
    """Compile and link the library if any source is newer than it.  checked
    = True makes the bounds-checked variant (-DLMG_BOUNDS_CHECK: failed index
    checks record a status word and skip the access) as
    liblmg_gb300_checked.so, from objects of its own."""
    objdir = OBJ.parent / "_build_checked" if checked else OBJ
    lib = LIB.with_name("liblmg_gb300_checked.so") if checked else LIB
    extra = ["-DLMG_BOUNDS_CHECK"] if checked else []
    objdir.mkdir(exist_ok=True)
    if force:
        for p in objdir.glob("*.o"):
            p.unlink()
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        errs = [e for e in ex.map(lambda u: _compile(u[0], u[1] + extra, u[2], objdir), UNITS)
                if e]
    if errs:
        raise RuntimeError("libmobility_gb300 build failed:\n" + "\n".join(errs))
    objs = [objdir / u[2] for u in UNITS]
    if force or not lib.exists() or any(o.stat().st_mtime > lib.stat().st_mtime for o in objs):
        cmd = [_nvcc(), "-shared", *ARCH, "-cudart", "static", "-o", str(lib),
               *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("libmobility_gb300 link failed:\n" + r.stdout + r.stderr)
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, checked="--checked" in sys.argv)
