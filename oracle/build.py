"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles this directory's own code: the FP64 C
  restatement ``rpy_oracle.c`` and the loader for the reference's GPU kernel
  ``ref_gpu_launcher.cpp`` into ``oracle/_build/``.  It works on any machine
  with gcc (the GPU machine included).
* ``build_reference()`` compiles libMobility's own sources, in place in the
  reference checkout, into ``oracle/_ref/``: the pair physics and the Lanczos
  solver for the CPU (both precisions) and the NBody "fast" CUDA kernel as an
  sm_103a cubin.  It runs only where the reference checkout exists; the GPU
  box uses the cubin made here (host objects made here are x86 and are not
  used there).

Nothing here is product code: libmobility_gb300 never imports this module.
"""
import os
import shutil
import subprocess
import sysconfig
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE = Path(os.environ.get("LMG_REFERENCE_SRC", "/root/reference"))
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(out: Path, *srcs: Path) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs)


def build_oracle(force: bool = False) -> None:
    """Compile the C oracle and the reference-kernel loader."""
    BUILD.mkdir(exist_ok=True)
    src = HERE / "rpy_oracle.c"
    out = BUILD / "liboracle.so"
    if force or _stale(out, src):
        _run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared",
              str(src), "-o", str(out), "-lpthread", "-lm"])
    src = HERE / "ref_gpu_launcher.cpp"
    out = BUILD / "libref_gpu_launcher.so"
    if force or _stale(out, src):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", str(src),
              f"-I{CUDA_HOME}/include", f"-L{CUDA_HOME}/lib64/stubs",
              f"-L{CUDA_HOME}/lib64", "-o", str(out), "-lcuda", "-lcudart"])


def _scipy_openblas():
    import scipy
    libs = Path(scipy.__file__).resolve().parent.parent / "scipy.libs"
    for p in sorted(libs.glob("libscipy_openblas*.so")):
        return p
    return None


def reference_available() -> bool:
    return (REFERENCE / "solvers/NBody/extra/hydrodynamicKernels.cuh").exists()


def build_reference(force: bool = False) -> None:
    """Compile the reference's own sources for the CPU and the GPU cubin."""
    if not reference_available():
        return
    REF_OUT.mkdir(exist_ok=True)
    drv = HERE / "ref_drivers.cpp"
    inc = [f"-I{CUDA_HOME}/include", f"-I{CUDA_HOME}/include/cccl",
           f"-I{REFERENCE}/include", f"-I{REFERENCE}"]
    hdrs = [REFERENCE / "solvers/NBody/extra/hydrodynamicKernels.cuh", drv]
    for suffix, flags in (("f", []), ("d", ["-DDOUBLE_PRECISION"])):
        out = REF_OUT / f"libref_pair_{suffix}.so"
        if force or _stale(out, *hdrs):
            _run(["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-fPIC",
                  "-shared", "-DREF_PAIR", *flags, *inc, str(drv), "-o", str(out)])
    blas = _scipy_openblas()
    if blas is not None:
        lhdrs = [REFERENCE / "include/lanczos/LanczosAlgorithm.cu", drv,
                 *sorted((HERE / "ref_shim").glob("*.h"))]
        for suffix, flags in (("f", []), ("d", ["-DDOUBLE_PRECISION"])):
            out = REF_OUT / f"libref_lanczos_{suffix}.so"
            if force or _stale(out, *lhdrs):
                _run(["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-fPIC",
                      "-shared", "-DREF_LANCZOS", *flags,
                      "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP",
                      f"-I{HERE / 'ref_shim'}", "-include",
                      str(HERE / "ref_shim/thrust_host.h"), *inc, str(drv),
                      "-o", str(out), str(blas), f"-Wl,-rpath,{blas.parent}"])
    nvcc = shutil.which("nvcc") or str(CUDA_HOME / "bin/nvcc")
    cu = HERE / "ref_gpu_kernels.cu"
    khdrs = [cu, REFERENCE / "solvers/NBody/extra/NbodyRPY.cu",
             REFERENCE / "solvers/NBody/extra/hydrodynamicKernels.cuh"]
    for suffix, flags in (("f", []), ("d", ["-DDOUBLE_PRECISION"])):
        out = REF_OUT / f"ref_nbody_{suffix}.cubin"
        if force or _stale(out, *khdrs):
            _run([nvcc, "-std=c++20", "--expt-relaxed-constexpr",
                  "-extended-lambda", "-cubin", "-O3",
                  "-gencode", "arch=compute_103a,code=sm_103a", *flags,
                  f"-I{REFERENCE}/include", f"-I{REFERENCE}", str(cu),
                  "-o", str(out)])


def build_all(force: bool = False) -> None:
    build_oracle(force)
    build_reference(force)


if __name__ == "__main__":
    build_all(force=True)
