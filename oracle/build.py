"""ORACLE build recipe (test infrastructure only).

Compiles ``oracle/neighconst.c`` (DP neighbor list), ``oracle/nepneigh.c`` (NEP neighbor
lists) and ``oracle/lammps_neigh.c`` (DP slots from a LAMMPS full list) into
``oracle/_build/libmatpl_oracle.so`` with gcc (``-fopenmp`` where available).
``-ffp-contract=off`` is required:
the restatements' floating-point order is the reference source order with no fused
multiply-add, on x86_64 and aarch64 alike.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmatpl_oracle.so")


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("neighconst.c", "nepneigh.c", "lammps_neigh.c")]
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(s) for s in srcs)):
        return LIB
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
           "-o", LIB, *srcs, "-lm"]
    # the centre-atom loops run in parallel with OpenMP where the compiler has it (results do
    # not depend on it: every atom's rows are computed in the serial order)
    if subprocess.call(cmd[:1] + ["-fopenmp"] + cmd[1:], stderr=subprocess.DEVNULL) != 0:
        subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
