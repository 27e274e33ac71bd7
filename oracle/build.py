"""ORACLE build recipe (test infrastructure only).

Compiles ``oracle/neighconst.c`` into ``oracle/_build/libmatpl_oracle.so`` with gcc.
``-ffp-contract=off`` is required: the restatement's floating-point order is the Fortran
source order with no fused multiply-add, on x86_64 and aarch64 alike.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libmatpl_oracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "neighconst.c")
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(src)):
        return LIB
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
           "-o", LIB, src, "-lm"]
    subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
