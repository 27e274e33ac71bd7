"""Build ``libmatpl_gb300.so`` (sm_103a only) in-tree with nvcc, and the ``CalcOps_cuda``
operator library ``libCalcOps_bind.so`` over it.

Each ``csrc/*.cu`` is compiled in parallel to an object file, then linked into one shared
library with the CUDA runtime linked statically (the library depends only on the driver).
``csrc/calcops_bind.cpp`` (the torch operator registrations, host code) is compiled with g++
against the installed libtorch at the same time and linked against both.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libmatpl_gb300.so")
OPS_LIB = os.path.join(OUT, "libCalcOps_bind.so")
OPS_SRC = os.path.join(SRC, "calcops_bind.cpp")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: matpl_gb300 needs the CUDA 13 toolkit to build")
    return cand


def _stale(lib: str, deps) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(d) > t for d in deps)


def _torch_flags():
    import torch
    from torch.utils import cpp_extension
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "include")
    inc = cpp_extension.include_paths() + [cuda_inc]
    cflags = ["-O2", "-fPIC", "-std=c++17",
              f"-D_GLIBCXX_USE_CXX11_ABI={int(torch._C._GLIBCXX_USE_CXX11_ABI)}"]
    libdir = cpp_extension.library_paths()[0]
    ldflags = [f"-L{libdir}", f"-Wl,-rpath,{libdir}", "-ltorch", "-ltorch_cpu", "-lc10",
               "-lc10_cuda"]
    return cflags + [f"-I{p}" for p in inc], ldflags


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(SRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(SRC, "*.cuh"))) + [
        os.path.join(os.path.dirname(HERE), "include", "matpl_gb300.h")]
    deps = sources + headers + [OPS_SRC, __file__]
    if not force and not _stale(LIB, deps) and not _stale(OPS_LIB, deps):
        return LIB
    nvcc = _nvcc()
    cflags, ldflags = _torch_flags()

    def compile_ops():
        obj = os.path.join(OUT, "calcops_bind.o")
        r = subprocess.run(["g++", *cflags, "-c", OPS_SRC, "-o", obj], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed on {OPS_SRC}:\n{r.stdout}\n{r.stderr}")
        return obj

    def compile_one(src):
        obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc, *ARCH, *FLAGS, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(sources) + 1)) as ex:
        ops_obj = ex.submit(compile_ops)
        objs = list(ex.map(compile_one, sources))
        ops_obj = ops_obj.result()
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    tmp = OPS_LIB + ".tmp"
    r = subprocess.run(["g++", "-shared", "-o", tmp, ops_obj, f"-L{OUT}", "-lmatpl_gb300",
                        "-Wl,-rpath,$ORIGIN", *ldflags], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of {OPS_LIB} failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OPS_LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
