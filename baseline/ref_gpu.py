"""The reference's own GPU code as a comparator: staging, build and a thin ctypes driver.

Two pieces of MatPL's CUDA code are built unmodified for sm_103a and timed / checked beside the
fused kernels on the same GPU:

* the LAMMPS NEP evaluator ``NEP3::compute_large_box_optim``
  (src/lmps/lammps-libtorch/MATPL/NEP_GPU/force/nep3.cu:551-810 with the kernels of
  nep3_large_box.cuh:46-800), four translation units (the NEP_GPU Makefile's CUDA_SOURCES:
  force/nep3.cu, utilities/error.cu, utilities/gpu_vector.cu, utilities/main_common.cu);
* the CalcOps_cuda force / virial launchers (src/op/kernel/calculateForce.cu,
  src/op/kernel/calculateVirial.cu, header src/op/include/calculate_force.h).

``stage()`` copies exactly those source files, keeping their relative paths, into the
git-ignored ``baseline/_ref/src`` (the reference tree exists only in the development
container; the staged copy travels with the working tree and is compiled where the GPU is).
``build()`` compiles them with nvcc (-std=c++17 -O3 as the NEP_GPU Makefile, one
``-gencode arch=compute_103a,code=sm_103a`` in place of its Pascal..Ada list; its unused
-lcublas -lcusolver are left out) together with ``baseline/ref_gpu_shim.cu`` into
``baseline/_ref/libmatpl_refgpu.so``.  ``load()`` returns the ctypes handle or None.

Nothing in the product links or imports this module: the benchmark and the comparator tests do.
"""
import ctypes
import os
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
STAGE = os.path.join(OUT, "src")
LIB = os.path.join(OUT, "libmatpl_refgpu.so")
SHIM = os.path.join(HERE, "ref_gpu_shim.cu")

NEP_DIR = os.path.join("src", "lmps", "lammps-libtorch", "MATPL", "NEP_GPU")
NEP_FILES = ["force/nep3.cu", "force/nep3.cuh", "force/nep3_large_box.cuh",
             "utilities/common.cuh", "utilities/error.cu", "utilities/error.cuh",
             "utilities/gpu_vector.cu", "utilities/gpu_vector.cuh", "utilities/main_common.cu",
             "utilities/main_common.cuh", "utilities/nep_utilities.cuh"]
NEP_UNITS = ["force/nep3.cu", "utilities/error.cu", "utilities/gpu_vector.cu",
             "utilities/main_common.cu"]
OP_DIR = os.path.join("src", "op")
OP_FILES = ["kernel/calculateForce.cu", "kernel/calculateVirial.cu", "include/calculate_force.h"]
OP_UNITS = ["kernel/calculateForce.cu", "kernel/calculateVirial.cu"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _reference_root():
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    from oracle.refpath import reference_root
    return reference_root()


def staged() -> bool:
    return all(os.path.exists(os.path.join(STAGE, NEP_DIR, f)) for f in NEP_FILES) and all(
        os.path.exists(os.path.join(STAGE, OP_DIR, f)) for f in OP_FILES)


def stage() -> bool:
    """Copy the listed reference files into baseline/_ref/src when the reference tree is
    present; returns whether a complete staged copy exists afterwards."""
    root = _reference_root()
    pairs = [(os.path.join(root, NEP_DIR, f), os.path.join(STAGE, NEP_DIR, f)) for f in NEP_FILES]
    pairs += [(os.path.join(root, OP_DIR, f), os.path.join(STAGE, OP_DIR, f)) for f in OP_FILES]
    if all(os.path.exists(s) for s, _ in pairs):
        for s, d in pairs:
            os.makedirs(os.path.dirname(d), exist_ok=True)
            if not os.path.exists(d) or os.path.getmtime(d) < os.path.getmtime(s):
                shutil.copy2(s, d)
    return staged()


def _nvcc():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else "nvcc"


def build(force: bool = False) -> str:
    """Stage (where the reference is present) and compile; returns the library path.  Raises
    FileNotFoundError when no staged copy exists."""
    if not stage():
        raise FileNotFoundError("reference GPU sources are not staged under baseline/_ref/src")
    srcs = [SHIM] + [os.path.join(STAGE, NEP_DIR, f) for f in NEP_FILES] + [
        os.path.join(STAGE, OP_DIR, f) for f in OP_FILES]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(s) for s in srcs):
        return LIB
    nep = os.path.join(STAGE, NEP_DIR)
    op = os.path.join(STAGE, OP_DIR)
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    base = [_nvcc(), "-std=c++17", "-O3", ARCH, "-Xcompiler=-fPIC"]
    nep_inc = [f"-I{nep}", f"-I{os.path.join(nep, 'force')}", f"-I{os.path.join(nep, 'utilities')}"]
    jobs = [(os.path.join(nep, u), nep_inc, f"nep_{i}.o") for i, u in enumerate(NEP_UNITS)]
    jobs += [(os.path.join(op, u), [f"-I{os.path.join(op, 'include')}"], f"op_{i}.o")
             for i, u in enumerate(OP_UNITS)]
    jobs.append((SHIM, nep_inc + [f"-I{os.path.join(op, 'include')}"], "shim.o"))

    def compile_one(job):
        src, inc, obj = job
        out = os.path.join(objdir, obj)
        subprocess.check_call(base + inc + ["-c", src, "-o", out])
        return out

    with ThreadPoolExecutor(len(jobs)) as ex:
        objs = list(ex.map(compile_one, jobs))
    tmp = LIB + ".tmp"
    subprocess.check_call([_nvcc(), "-shared", ARCH, "-o", tmp] + objs)
    os.replace(tmp, LIB)
    return LIB


_HANDLE = None


def load():
    """ctypes handle to the comparator library (built earlier), or None when it is absent."""
    global _HANDLE
    if _HANDLE is not None:
        return _HANDLE
    if not os.path.exists(LIB):
        return None
    lib = ctypes.CDLL(LIB)
    P, I = ctypes.c_void_p, ctypes.c_int
    lib.refnep_create.restype = P
    lib.refnep_create.argtypes = [ctypes.c_char_p, I]
    lib.refnep_destroy.restype = None
    lib.refnep_destroy.argtypes = [P]
    lib.refnep_capacity.restype = I
    lib.refnep_capacity.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I),
                                    ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    lib.refnep_compute.restype = I
    lib.refnep_compute.argtypes = [P, I, I, I, I, I, P, P, P, P, P, P, P, P]
    lib.refcalc_force.restype = I
    lib.refcalc_force.argtypes = [I, P, P, P, I, I, I, P, I, I]
    lib.refcalc_virial.restype = I
    lib.refcalc_virial.argtypes = [I, P, P, P, P, I, I, I, P, P, I, I]
    _HANDLE = lib
    return lib


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def pair_counts(system, rc: float) -> np.ndarray:
    """Listed pairs per local atom that the evaluator's filter keeps for cutoff rc: the squared
    distance summed in FP64, rounded to FP32 and compared with rc*rc formed in FP32
    (find_neighbor_list_large_box, nep3_large_box.cuh:70-80)."""
    x = system["x"]
    n = system["nlocal"]
    rows = np.repeat(np.arange(n), system["numneigh"])
    d = x[system["jflat"]] - x[rows]
    d2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]).astype(np.float32)
    rc32 = np.float32(rc)
    keep = d2 < np.float32(rc32 * rc32)
    return np.bincount(rows[keep], minlength=n)


class RefNEP:
    """The reference GPU NEP evaluator on one LAMMPS-style system (local atoms + ghost images,
    full neighbor lists), driven as PairMATPL::compute drives it: type indices, the list padded
    to [inum, NM] and SoA positions packed once (convert_dim, pair_matpl.cpp:730-760), then one
    ``compute`` per step."""

    def __init__(self, nep_text: str, system, types0: np.ndarray, device: int = 0):
        lib = load()
        if lib is None:
            raise FileNotFoundError("comparator library not built")
        self.lib = lib
        fd, path = tempfile.mkstemp(suffix=".nep.txt")
        with os.fdopen(fd, "w") as f:
            f.write(nep_text)
        try:
            self.h = lib.refnep_create(path.encode(), device)
        finally:
            os.remove(path)
        if not self.h:
            raise RuntimeError("refnep_create failed")
        mr, ma = ctypes.c_int(), ctypes.c_int()
        rr, ra = ctypes.c_float(), ctypes.c_float()
        lib.refnep_capacity(self.h, ctypes.byref(mr), ctypes.byref(ma), ctypes.byref(rr),
                            ctypes.byref(ra))
        self.capacity = (mr.value, ma.value)
        cr, ca = pair_counts(system, rr.value), pair_counts(system, ra.value)
        self.max_pairs = (int(cr.max()), int(ca.max()))
        # the evaluator writes its lists without a bound and sorts them one thread per entry
        if cr.max() > mr.value or ca.max() > ma.value or max(mr.value, ma.value) > 1024:
            self.close()
            raise ValueError(f"pairs per atom {self.max_pairs} exceed the evaluator's list "
                             f"capacities {self.capacity} (or a capacity exceeds 1024)")
        n, nall = system["nlocal"], system["nlocal"] + system["nghost"]
        self.n, self.nall = n, nall
        self.nm = int(system["numneigh"].max())
        self.itype = np.ascontiguousarray(types0, dtype=np.int32)
        assert self.itype.shape == (nall,)
        self.ilist = np.ascontiguousarray(system["ilist"], dtype=np.int32)
        self.numneigh = np.ascontiguousarray(system["numneigh"], dtype=np.int32)
        fn = np.zeros((n, self.nm), dtype=np.int32)
        rows = np.repeat(np.arange(n), self.numneigh)
        cols = np.arange(rows.size) - np.repeat(system["jstart"][:-1], self.numneigh)
        fn[rows, cols] = system["jflat"]
        self.firstneigh = fn
        self.pos = np.ascontiguousarray(system["x"].T.reshape(-1))
        self.ei = np.zeros(n)
        self.force = np.zeros(3 * nall)
        self.virial = np.zeros(6)

    def compute(self, build_neighbor: bool = True):
        """Ei [n], force [nall, 3] (local and ghost rows), virial [6] (xx yy zz xy xz yz)."""
        rc = self.lib.refnep_compute(
            self.h, int(build_neighbor), self.nall, self.n, self.n, self.nm, _ptr(self.itype),
            _ptr(self.ilist), _ptr(self.numneigh), _ptr(self.firstneigh), _ptr(self.pos),
            _ptr(self.ei), _ptr(self.force), _ptr(self.virial))
        if rc != 0:
            raise RuntimeError(f"reference NEP evaluator: CUDA error {rc}")
        return self.ei, self.force.reshape(3, self.nall).T, self.virial

    def close(self):
        if getattr(self, "h", None):
            self.lib.refnep_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
