"""Build the CUDA library ``libpylops_gb300.so`` in-tree with nvcc for sm_103a.

The library holds every kernel of the package and its C ABI
(``include/kirchhoff_gb300.h``).  Translation units compile in parallel; the
result lands in ``pylops_gb300/_lib/``.
"""

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIBNAME = "libpylops_gb300.so"
SOURCES = ["kirchhoff_kernels.cu", "kirchhoff_capi.cu", "solver.cu", "eikonal.cpp", "forward_static.cu", "batch.cu", "gemm_tcgen05.cu", "unet_kernels.cu", "nsconv2d.cu", "tables.cu"]
HEADERS = ["kgb_internal.h", "fir.cuh", "fixed_acc.cuh", "tma.cuh", "dfacc.cuh", os.path.join("..", "..", "include", "kirchhoff_gb300.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2,-fopenmp"]


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the pylops_gb300 CUDA library cannot be built")


def _stale() -> bool:
    out = lib_path()
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    deps = [os.path.join(CSRC, s) for s in SOURCES] + [os.path.join(CSRC, h) for h in HEADERS]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if stale) and return the path of the shared library."""
    if not force and not _stale():
        return lib_path()
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    objs = []

    def _one(src):
        obj = os.path.join(LIBDIR, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_one, SOURCES))
    tmp = lib_path() + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path())
    for o in objs:
        os.remove(o)
    return lib_path()


if __name__ == "__main__":
    print(build(force=True, verbose=True))
