"""Recipe that compiles the reference's own CPU operator library (test infrastructure only).

MatPL registers its CPU operators with ``TORCH_LIBRARY(CalcOps_cpu, m)``
(src/op/src/CalcOps_bind_cpu.cpp:6-13) from three translation units
(src/op/cmake/cpu/CMakeLists.txt:2-6): CalcOps_cpu.cpp, cpu_calculate_nepneighbor.cpp and
nep_cpu.cpp.  This script compiles those files where they lie in the reference tree, with g++
against the installed libtorch, into ``oracle/_ref/libCalcOps_bind_cpu.so``; nothing is copied
and the reference's own build system is not run.  Loading the result with
``torch.ops.load_library`` exposes ``torch.ops.CalcOps_cpu.calculate_neighbor``,
``calculate_maxneigh`` and ``calculate_descriptor``, which the NEP golden-fixture script
(tests/golden/make_nep_golden.py) runs to pin the NEP oracle.

The reference sources exist only in the development container, so this recipe is never part of
the shipped build; ``-ffp-contract=off`` keeps the arithmetic free of fused multiply-adds, as a
default x86_64 build of the reference is.
"""
import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libCalcOps_bind_cpu.so")
sys.path.insert(0, os.path.dirname(HERE))
from oracle.refpath import reference_root  # noqa: E402

REF_OP = os.environ.get("MATPL_REFERENCE_OP_DIR") or os.path.join(reference_root(), "src", "op")
SOURCES = ["CalcOps_cpu.cpp", "cpu_calculate_nepneighbor.cpp", "nep_cpu.cpp",
           "CalcOps_bind_cpu.cpp"]


def available() -> bool:
    return all(os.path.exists(os.path.join(REF_OP, "src", s)) for s in SOURCES)


def build(force: bool = False) -> str:
    if not available():
        raise FileNotFoundError(f"reference operator sources not found under {REF_OP}")
    if not force and os.path.exists(LIB):
        return LIB
    from torch.utils import cpp_extension
    os.makedirs(OUT_DIR, exist_ok=True)
    inc = cpp_extension.include_paths()
    flags = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-std=c++17",
             "-DTORCH_EXTENSION_NAME=CalcOps_bind_cpu", "-DTORCH_API_INCLUDE_EXTENSION_H"]
    flags += [f"-I{p}" for p in inc] + [f"-I{sysconfig.get_paths()['include']}",
                                         f"-I{os.path.join(REF_OP, 'include')}"]

    def compile_one(src):
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        subprocess.check_call(["g++", *flags, "-c", os.path.join(REF_OP, "src", src), "-o", obj])
        return obj

    with ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    libdir = cpp_extension.library_paths()[0]
    subprocess.check_call(["g++", "-shared", "-o", LIB, *objs, f"-L{libdir}",
                           f"-Wl,-rpath,{libdir}", "-ltorch", "-ltorch_cpu", "-lc10"])
    for o in objs:
        os.remove(o)
    return LIB


def load():
    """Build if needed and register ``torch.ops.CalcOps_cpu``."""
    import torch
    torch.ops.load_library(build())
    return torch.ops.CalcOps_cpu


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
